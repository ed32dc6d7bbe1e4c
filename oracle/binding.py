"""ctypes binding of the CPU oracle (oracle/_build/libpforacle.so).

ORACLE / TEST INFRASTRUCTURE ONLY: imported by tests, by the smoke check and
by the benchmark's CPU-baseline leg, never by the product package.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent
LIB = HERE / "_build" / "libpforacle.so"
REFEMU_LIB = HERE / "_ref" / "librefemu.so"


def build(force: bool = False) -> Path:
    """Compiles the oracle with gcc (portable flags, no FMA contraction so x86
    and Arm hosts give the same bits)."""
    src = HERE / "pf_oracle.c"
    if force or not LIB.exists() or LIB.stat().st_mtime < max(src.stat().st_mtime,
                                                              (ROOT / "include" / "pfgpu.h").stat().st_mtime,
                                                              (HERE / "pf_oracle.h").stat().st_mtime):
        LIB.parent.mkdir(parents=True, exist_ok=True)
        tmp = LIB.with_suffix(f".{os.getpid()}.tmp.so")
        subprocess.run(["gcc", "-O3", "-fopenmp", "-fPIC", "-shared", "-std=c11", "-ffp-contract=off",
                        f"-I{ROOT / 'include'}", str(src), "-o", str(tmp), "-lm"], check=True)
        os.replace(tmp, LIB)
    return LIB


def reference_dir() -> Path:
    """Where the reference's source tree is looked for: $PF_REFERENCE_DIR,
    else a `reference` directory beside this checkout."""
    env = os.environ.get("PF_REFERENCE_DIR")
    return Path(env) if env else ROOT.parent / "reference"


def build_refemu() -> Path | None:
    """Builds oracle/_ref/librefemu.so from the reference tree when present."""
    script = HERE / "refemu" / "build_refemu.sh"
    subprocess.run(["sh", str(script)], check=True, env=dict(os.environ, REF_DIR=str(reference_dir())))
    return REFEMU_LIB if REFEMU_LIB.exists() else None


_lib = None


def lib():
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(str(LIB))
        vp, dp, ip = C.c_void_p, C.POINTER(C.c_double), C.POINTER(C.c_int)
        L.pfo_create.restype = vp
        L.pfo_create.argtypes = [vp, C.c_int]
        L.pfo_destroy.argtypes = [vp]
        L.pfo_step.restype = C.c_int
        L.pfo_step.argtypes = [vp, C.c_int]
        L.pfo_set_threads.argtypes = [C.c_int]
        L.pfo_get_lattice.argtypes = [vp, dp, dp, dp, dp, dp]
        L.pfo_get_elements.argtypes = [vp, dp, dp, dp, dp, dp, dp]
        L.pfo_get_bonds.argtypes = [vp, ip, ip, ip]
        L.pfo_get_fibrin.argtypes = [vp, dp, dp, dp, dp, dp]
        L.pfo_get_membrane.argtypes = [vp, dp, dp]
        L.pfo_conservation.argtypes = [vp, dp]
        L.pfo_get_cells.restype = C.c_int
        L.pfo_get_cells.argtypes = [vp, ip, ip, ip]
        L.pfo_step_count.restype = C.c_longlong
        L.pfo_step_count.argtypes = [vp]
        L.pfo_receptor_uniforms.argtypes = [C.c_uint64, C.c_int64, C.c_int64, dp]
        L.pfo_detach_uniform.restype = C.c_double
        L.pfo_detach_uniform.argtypes = [C.c_uint64, C.c_int64]
        L.pfo_philox4x32.argtypes = [C.POINTER(C.c_uint32), C.POINTER(C.c_uint32), C.POINTER(C.c_uint32)]
        L.pfo_ibm_phi.restype = C.c_double
        L.pfo_ibm_phi.argtypes = [C.c_double]
        L.pfo_feq.argtypes = [C.c_double, dp, C.c_double, dp]
        L.pfo_wlc_force.restype = C.c_double
        L.pfo_wlc_force.argtypes = [C.c_double, C.c_double, C.c_double]
        _lib = L
    return _lib


def _p(a, t=C.c_double):
    return a.ctypes.data_as(C.POINTER(t))


def set_threads(n: int):
    lib().pfo_set_threads(int(n))


def receptor_uniforms(seed: int, step: int, receptor: int) -> np.ndarray:
    out = np.zeros(2)
    lib().pfo_receptor_uniforms(seed, step, receptor, _p(out))
    return out


def detach_uniform(seed: int, step: int) -> float:
    return lib().pfo_detach_uniform(seed, step)


def philox4x32(ctr, key) -> np.ndarray:
    c = np.asarray(ctr, dtype=np.uint32)
    k = np.asarray(key, dtype=np.uint32)
    o = np.zeros(4, dtype=np.uint32)
    lib().pfo_philox4x32(_p(c, C.c_uint32), _p(k, C.c_uint32), _p(o, C.c_uint32))
    return o


def feq(rho: float, u, C_: float) -> np.ndarray:
    uu = np.asarray(u, dtype=np.float64)
    out = np.zeros(19)
    lib().pfo_feq(rho, _p(uu), C_, _p(out))
    return out


class Oracle:
    """One CPU FP64 simulation of a Scene."""

    def __init__(self, scene, brute: bool = False):
        self.scene = scene
        self._c = scene.to_c()
        self.h = lib().pfo_create(C.byref(self._c), 1 if brute else 0)
        if not self.h:
            raise RuntimeError("pfo_create failed")

    def close(self):
        if self.h:
            lib().pfo_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def step(self, n: int = 1) -> int:
        return lib().pfo_step(self.h, int(n))

    @property
    def steps(self) -> int:
        return lib().pfo_step_count(self.h)

    def lattice(self):
        N = self.scene.n_nodes
        fIN, fOUT = np.zeros((19, N)), np.zeros((19, N))
        rho, u, F = np.zeros(N), np.zeros((3, N)), np.zeros((3, N))
        lib().pfo_get_lattice(self.h, _p(fIN), _p(fOUT), _p(rho), _p(u), _p(F))
        return dict(fIN=fIN, fOUT=fOUT, rho=rho, u=u, F=F)

    def elements(self):
        PE = self.scene.n_platelets * self.scene.n_elem
        X, Y, RY, Z = (np.zeros(PE) for _ in range(4))
        V, F = np.zeros((3, PE)), np.zeros((3, PE))
        lib().pfo_get_elements(self.h, _p(X), _p(Y), _p(RY), _p(Z), _p(V), _p(F))
        return dict(X=X, Y=Y, RY=RY, Z=Z, V=V, F=F)

    def bonds(self):
        sc = self.scene
        st = np.zeros((sc.n_platelets, sc.n_rec, 3), dtype=np.int32)
        vwf = np.zeros((4, sc.ny, sc.nx), dtype=np.int32)
        tot = C.c_int(0)
        lib().pfo_get_bonds(self.h, _p(st, C.c_int), _p(vwf, C.c_int), C.byref(tot))
        return dict(rec_state=st, vwf=vwf, total=tot.value)

    def fibrin(self):
        M = self.scene.n_fib
        X, Y, Z = np.zeros(M), np.zeros(M), np.zeros(M)
        V, F = np.zeros((3, M)), np.zeros((3, M))
        lib().pfo_get_fibrin(self.h, _p(X), _p(Y), _p(Z), _p(V), _p(F))
        return dict(X=X, Y=Y, Z=Z, V=V, F=F)

    def membrane(self):
        sc = self.scene
        SV = np.zeros((sc.n_platelets, 2))
        km = np.zeros((sc.n_platelets, sc.n_membrane))
        lib().pfo_get_membrane(self.h, _p(SV), _p(km))
        return dict(S_V=SV, km=km)

    def conservation(self):
        out = np.zeros(4)
        lib().pfo_conservation(self.h, _p(out))
        return out

    def cells(self):
        PE = self.scene.n_platelets * self.scene.n_elem
        cell_of = np.zeros(PE, dtype=np.int32)
        order = np.zeros(PE, dtype=np.int32)
        nc = np.zeros(3, dtype=np.int32)
        lib().pfo_get_cells(self.h, _p(cell_of, C.c_int), _p(order, C.c_int), _p(nc, C.c_int))
        return cell_of, order, nc


def wlc_force(l0: float, l: float, mass: float) -> float:
    """The oracle's worm-like-chain link force (fiber.cpp:710-733)."""
    return float(lib().pfo_wlc_force(l0, l, mass))
