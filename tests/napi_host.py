"""A Python host for the Node-API addon, standing in for Node in the tests.

TEST INFRASTRUCTURE. Builds tests/napi/napi_stub.c (a minimal Node-API
implementation) and, for CPU tests, tests/napi/fake_caustic.c (a recording
stand-in for libcaustic_gb300) plus the addon linked against it, all with gcc
into tests/_build/. `NodeHost` loads an addon through the stub the way Node
does (napi_register_module_v1) and converts Python values to and from the
stub's JavaScript values: dicts become objects, numpy arrays typed arrays
(borrowed, not copied), and a pending exception is raised as `JsError`.
"""
from __future__ import annotations

import ctypes as C
import os
import pathlib
import shutil
import subprocess
import threading

import numpy as np

ROOT = pathlib.Path(__file__).resolve().parent.parent
NAPI_SRC = ROOT / "caustic-tracer_gb300" / "napi"
TEST_SRC = ROOT / "tests" / "napi"
OUT = ROOT / "tests" / "_build"
STUB = OUT / "libnapi_stub.so"
FAKE = OUT / "libct_fake.so"
FAKE_ADDON = OUT / "caustic_addon_fake.node"
REAL_ADDON = ROOT / "caustic-tracer_gb300" / "_build" / "caustic_addon.node"

TYPED = {np.dtype(np.int8): 0, np.dtype(np.uint8): 1, np.dtype(np.int16): 3, np.dtype(np.uint16): 4,
         np.dtype(np.int32): 5, np.dtype(np.uint32): 6, np.dtype(np.float32): 7, np.dtype(np.float64): 8}
DTYPE = {v: k for k, v in TYPED.items()}
K_UNDEF, K_NULL, K_BOOL, K_NUM, K_STR, K_OBJ, K_ABUF, K_TYPED, K_EXT, K_FUNC = range(10)
ERROR_KINDS = {1: "Error", 2: "TypeError", 3: "RangeError"}
_lock = threading.Lock()
_stub = None


class JsError(Exception):
    """An exception the addon threw: kind (Error, TypeError, RangeError), code and message."""

    def __init__(self, kind: str, code: str, message: str):
        super().__init__(f"{kind} [{code}]: {message}")
        self.kind, self.code, self.message = kind, code, message


def _cc(args):
    cc = shutil.which("gcc") or shutil.which("cc")
    res = subprocess.run([cc, *args], capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"{' '.join(args)}\n{res.stdout}\n{res.stderr}")


def _stale(out: pathlib.Path, deps) -> bool:
    return not out.exists() or any(pathlib.Path(d).stat().st_mtime > out.stat().st_mtime for d in deps)


def build() -> None:
    """Compiles the stub, the fake library and the addon against the fake (idempotent)."""
    OUT.mkdir(parents=True, exist_ok=True)
    inc = [f"-I{NAPI_SRC}", f"-I{ROOT / 'include'}"]
    common = ["-std=c11", "-O1", "-g", "-fPIC", "-shared", "-Wall", "-Wextra", "-Werror", *inc]
    if _stale(STUB, [TEST_SRC / "napi_stub.c", NAPI_SRC / "node_api_min.h"]):
        _cc([*common, str(TEST_SRC / "napi_stub.c"), "-o", str(STUB), "-ldl"])
    if _stale(FAKE, [TEST_SRC / "fake_caustic.c", ROOT / "include" / "caustic.h"]):
        _cc([*common, str(TEST_SRC / "fake_caustic.c"), "-o", str(FAKE)])
    if _stale(FAKE_ADDON, [NAPI_SRC / "caustic_addon.c", NAPI_SRC / "node_api_min.h", FAKE]):
        _cc([*common, str(NAPI_SRC / "caustic_addon.c"), "-o", str(FAKE_ADDON), f"-L{OUT}", "-lct_fake",
             "-Wl,-rpath,$ORIGIN", "-lm"])


def stub() -> C.CDLL:
    """The Node-API stub, loaded with RTLD_GLOBAL so addons resolve napi_* against it."""
    global _stub
    with _lock:
        if _stub is None:
            build()
            L = C.CDLL(str(STUB), mode=os.RTLD_GLOBAL | os.RTLD_NOW)
            P = C.c_void_p
            sig = {
                "stub_env_new": (P, []), "stub_env_free": (None, [P]), "stub_collect": (C.c_int, [P]),
                "stub_undefined": (P, [P]), "stub_null": (P, [P]), "stub_bool": (P, [P, C.c_int]),
                "stub_number": (P, [P, C.c_double]), "stub_string": (P, [P, C.c_char_p]),
                "stub_object": (P, [P]), "stub_set": (C.c_int, [P, P, C.c_char_p, P]),
                "stub_typed": (P, [P, C.c_int, P, C.c_size_t]), "stub_kind": (C.c_int, [P]),
                "stub_number_of": (C.c_double, [P]),
                "stub_typed_info": (C.c_int, [P, C.POINTER(C.c_int), C.POINTER(C.c_void_p), C.POINTER(C.c_size_t)]),
                "stub_finalized": (C.c_int, [P]),
                "stub_load": (P, [P, C.c_char_p, C.c_char_p, C.c_size_t]),
                "stub_call": (P, [P, P, C.c_char_p, C.c_size_t, C.POINTER(P)]),
                "stub_take_exception": (C.c_int, [P, C.c_char_p, C.c_size_t, C.c_char_p, C.c_size_t]),
            }
            for name, (res, args) in sig.items():
                fn = getattr(L, name)
                fn.restype, fn.argtypes = res, args
            _stub = L
    return _stub


def fake() -> C.CDLL:
    """The recording fake library (the same loaded object the fake addon uses)."""
    build()
    return C.CDLL(str(FAKE))


class NodeHost:
    """One Node-API environment with one loaded addon."""

    def __init__(self, addon_path: pathlib.Path):
        self.S = stub()
        self.env = self.S.stub_env_new()
        self._keep = []  # numpy arrays backing typed arrays stay alive with the env
        err = C.create_string_buffer(512)
        self.exports = self.S.stub_load(self.env, str(addon_path).encode(), err, 512)
        if not self.exports:
            raise RuntimeError(f"cannot load {addon_path}: {err.value.decode()}")

    def close(self):
        if self.env:
            self.S.stub_env_free(self.env)
            self.env = None
            self._keep.clear()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    # Python -> JavaScript
    def js(self, x):
        S, env = self.S, self.env
        if isinstance(x, JsValue):
            return x.handle
        if x is None:
            return S.stub_undefined(env)
        if isinstance(x, bool):
            return S.stub_bool(env, int(x))
        if isinstance(x, (int, float, np.integer, np.floating)):
            return S.stub_number(env, float(x))
        if isinstance(x, str):
            return S.stub_string(env, x.encode())
        if isinstance(x, np.ndarray):
            if x.dtype not in TYPED or not x.flags.c_contiguous:
                raise TypeError(f"no typed array for {x.dtype}")
            self._keep.append(x)
            return S.stub_typed(env, TYPED[x.dtype], C.c_void_p(x.ctypes.data), x.size)
        if isinstance(x, dict):
            o = S.stub_object(env)
            for k, v in x.items():
                S.stub_set(env, o, k.encode(), self.js(v))
            return o
        raise TypeError(f"cannot pass {type(x)}")

    def call(self, name: str, *args):
        """exports[name](*args); returns a JsValue, or raises JsError."""
        handles = (C.c_void_p * max(1, len(args)))(*[self.js(a) for a in args])
        r = self.S.stub_call(self.env, self.exports, name.encode(), len(args), handles)
        code, msg = C.create_string_buffer(96), C.create_string_buffer(1024)
        kind = self.S.stub_take_exception(self.env, code, 96, msg, 1024)
        if kind:
            raise JsError(ERROR_KINDS.get(kind, "Error"), code.value.decode(), msg.value.decode())
        return JsValue(self, r)

    def collect(self) -> int:
        """Runs the finalizers of unreleased externals (garbage collection); returns how many ran."""
        return self.S.stub_collect(self.env)


class JsValue:
    def __init__(self, host: NodeHost, handle):
        self.host, self.handle = host, handle

    @property
    def kind(self) -> int:
        return self.host.S.stub_kind(self.handle)

    def array(self) -> np.ndarray:
        """A copy of a typed array's elements."""
        t, d, n = C.c_int(), C.c_void_p(), C.c_size_t()
        if not self.host.S.stub_typed_info(self.handle, C.byref(t), C.byref(d), C.byref(n)):
            raise TypeError("not a typed array")
        dt = DTYPE[t.value]
        if n.value == 0:
            return np.zeros(0, dt)
        buf = (C.c_char * (n.value * dt.itemsize)).from_address(d.value)
        return np.frombuffer(buf, dtype=dt).copy()


def packed_scene_js(packed) -> dict:
    """A caustic.PackedScene as the reference's PackedScene object (pack.ts:46-59)."""
    sky = packed.sky
    if getattr(sky, "kind", "none") == "gradient":
        col = lambda c: {"r": c[0], "g": c[1], "b": c[2]}  # noqa: E731
        js_sky = {"kind": "gradient", "zenith": col(sky.zenith), "horizon": col(sky.horizon), "strength": sky.strength}
    else:
        js_sky = {"kind": "none"}
    return {"prims": packed.prims, "primCount": packed.prim_count, "nodes": packed.nodes,
            "nodeCount": packed.node_count, "mats": packed.mats, "matCount": packed.mat_count,
            "lights": packed.lights, "primObject": packed.prim_object, "sky": js_sky}


def frame_js(frame) -> dict:
    """A caustic.CameraFrame as the reference's CameraFrame object (camera.ts:8-20)."""
    v = lambda a: {"x": a[0], "y": a[1], "z": a[2]}  # noqa: E731
    return {"origin": v(frame.origin), "right": v(frame.right), "up": v(frame.up), "forward": v(frame.forward),
            "tanHalfFov": frame.tan_half_fov, "aspect": frame.aspect, "lensRadius": frame.lens_radius,
            "focusDistance": frame.focus_distance}
