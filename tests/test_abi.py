"""The C-ABI library loads and exports every function include/*.h declares."""
import pathlib
import re

import numpy as np

ROOT = pathlib.Path(__file__).resolve().parent.parent


def declared_functions():
    names = set()
    for header in (ROOT / "include").glob("*.h"):
        text = re.sub(r"/\*.*?\*/", "", header.read_text(), flags=re.S)
        for m in re.finditer(r"^[A-Za-z_][\w \*]*?\b(ct_\w+)\s*\(", text, flags=re.M):
            names.add(m.group(1))
    return names


def test_library_exports_every_declared_symbol(native_lib):
    names = declared_functions()
    assert "ct_trace_closest" in names and "ct_render_image" in names
    missing = [n for n in sorted(names) if not hasattr(native_lib, n)]
    assert not missing, missing


def test_python_signatures_cover_header(native_lib):
    from caustic import _abi

    assert declared_functions() <= set(_abi.SIGNATURES), declared_functions() - set(_abi.SIGNATURES)


def test_abi_version_and_struct_sizes(native_lib):
    import ctypes as C

    from caustic import _abi

    assert native_lib.ct_abi_version() == 1
    assert C.sizeof(_abi.ct_camera_frame) == 16 * 8
    assert C.sizeof(_abi.ct_render_options) == 7 * 4
    assert C.sizeof(_abi.ct_sky) == 8 + 7 * 8


def test_rng_stream_matches_python_and_oracle(native_lib, oracle):
    from caustic import Rng

    for seed in (0, 1, 42, 1234, 0xFFFFFFFF):
        r = Rng(seed)
        scalar = [r.next() for _ in range(50)]
        assert np.array_equal(Rng(seed).draw(50), np.array(scalar))
        assert np.array_equal(oracle.rng_stream(seed, 50), np.array(scalar))
    r = Rng(9)
    head = r.draw(7)
    tail = r.draw(5)
    assert np.array_equal(np.concatenate([head, tail]), oracle.rng_stream(9, 12))


def test_seed_for_and_pcg_match_oracle(oracle):
    from caustic import pcg_hash, seed_for

    for x in (0, 1, 7, 12345, 0x9E3779B9, 0xFFFFFFFF):
        assert pcg_hash(x) == oracle.lib().or_pcg_hash(x)
        for f in (0, 1, 7919, 100000):
            assert seed_for(x, f) == oracle.lib().or_seed_for(x, f)


def test_camera_frame_matches_oracle(oracle):
    import caustic as ct

    for cam in (ct.CORNELL_BOX.camera, ct.camera_at((4.2, 1.6, 4.6), (0, 0.35, 0), 30, 0.02, 6.2),
                ct.camera_at((12, 2.2, 3.2), (0, 0.55, 0), 22, 0.06, 10.5)):
        for aspect in (1.0, 1.5, 16 / 9):
            mine = ct.camera_frame(cam, aspect).struct()
            want = oracle.camera_frame(oracle.settings_struct(cam), aspect)
            for f in ("origin", "right", "up", "forward"):
                assert list(getattr(mine, f)) == list(getattr(want, f)), f
            for f in ("tan_half_fov", "aspect", "lens_radius", "focus_distance"):
                assert getattr(mine, f) == getattr(want, f), f


def test_scene_create_rejects_malformed_arrays(native_lib):
    """Host-side validation turns bad indices into CT_ERR_INVALID_ARGUMENT (no device needed)."""
    import ctypes as C

    import caustic as ct

    ps = ct.pack_scene(ct.CORNELL_BOX)
    bad = ct.PackedScene(ps.prims.copy(), ps.prim_count, ps.nodes.copy(), ps.node_count, ps.mats.copy(),
                         ps.mat_count, np.array([99], np.int32), ps.prim_object.copy(), ps.sky, ps.order)
    h = C.c_void_p()
    v = bad.view()
    assert native_lib.ct_scene_create(C.byref(v), C.byref(h)) == 1
    assert b"lights" in native_lib.ct_last_error()
    bad2 = ct.PackedScene(ps.prims.copy(), ps.prim_count, ps.nodes.copy(), ps.node_count, ps.mats.copy(),
                          ps.mat_count, ps.lights.copy(), ps.prim_object.copy(), ps.sky, ps.order)
    bad2.nodes[3] = 5  # root skip link no longer ends the tree
    v2 = bad2.view()
    assert native_lib.ct_scene_create(C.byref(v2), C.byref(h)) == 1
    assert b"skip" in native_lib.ct_last_error()


def test_large_scene_validation_on_worker_threads_reports_here(native_lib):
    """Scenes of 50,000 primitives or more check their values on worker threads
    beside the tree check; a failure still comes back as this call's status and
    this thread's ct_last_error message (no device needed)."""
    import ctypes as C

    import caustic as ct

    ps = ct.pack_scene(ct.triangle_soup(60_000, seed=3))
    h = C.c_void_p()
    cases = []
    prims = ps.prims.copy()
    prims[16 * 1234 + 5] = np.nan
    cases.append((ct.PackedScene(prims, ps.prim_count, ps.nodes, ps.node_count, ps.mats, ps.mat_count, ps.lights,
                                 ps.prim_object, ps.sky, ps.order), b"non-finite"))
    nodes = ps.nodes.copy()
    nodes[8 * 77 + 1] = np.inf
    cases.append((ct.PackedScene(ps.prims, ps.prim_count, nodes, ps.node_count, ps.mats, ps.mat_count, ps.lights,
                                 ps.prim_object, ps.sky, ps.order), b"not finite"))
    obj = ps.prim_object.copy()
    obj[59_999] = 7
    cases.append((ct.PackedScene(ps.prims, ps.prim_count, ps.nodes, ps.node_count, ps.mats, ps.mat_count, ps.lights,
                                 obj, ps.sky, ps.order), b"prim_object"))
    for bad, msg in cases:
        v = bad.view()
        assert native_lib.ct_scene_create(C.byref(v), C.byref(h)) == 1
        assert msg in native_lib.ct_last_error(), native_lib.ct_last_error()
