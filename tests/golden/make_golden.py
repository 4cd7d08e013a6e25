"""Regenerates the golden fixtures in this folder from the reference checkout.

cornell.ppm is the reference's own committed render (out/cornell.ppm of
caustic-tracer): `npm run render:cpu` with its defaults, i.e.
renderCornellReference(96, 64, 16) -> 16 spp, ACES, NEE on, Russian roulette
on, 8 bounces, seed 1 (scripts/render-cpu.ts:13-22, src/tracer/reference.ts:20-43).
It is copied verbatim, and its SHA-256 is recorded in cornell.ppm.sha256.

Usage: python tests/golden/make_golden.py /path/to/caustic-tracer
"""
import hashlib
import pathlib
import shutil
import sys


def main() -> None:
    if len(sys.argv) != 2:
        sys.exit("usage: python tests/golden/make_golden.py /path/to/caustic-tracer")
    ref = pathlib.Path(sys.argv[1])
    here = pathlib.Path(__file__).resolve().parent
    src = ref / "out" / "cornell.ppm"
    dst = here / "cornell.ppm"
    shutil.copyfile(src, dst)
    digest = hashlib.sha256(dst.read_bytes()).hexdigest()
    (here / "cornell.ppm.sha256").write_text(digest + "  cornell.ppm\n")
    print("wrote", dst, digest)


if __name__ == "__main__":
    main()
