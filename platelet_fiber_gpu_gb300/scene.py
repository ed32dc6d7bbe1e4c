"""Host-side description of one coupled simulation (`pf_scene` of pfgpu.h).

`Scene` owns numpy arrays in the layouts pfgpu.h documents and produces the
ctypes struct that both the CUDA library and the CPU oracle read.
`reference_params` restates the reference driver's parameter table
(gpuSEM_LB.c:1206-1233) in float32, like the constant array it is uploaded
to (semLB.cu:46).
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass, field

import numpy as np

BC_PERIODIC, BC_BOUNCEBACK, BC_ZOUHE_SHEAR = 0, 1, 2
# velocity inlet at y=0 / outlet at y=ny-1 with the shear profile (y only)
BC_INOUT = 3
PREC_FP64, PREC_FP32, PREC_FP16 = 0, 1, 2
BOND_BELL, BOND_CONSTANT = 0, 1
FIB_HOOKE, FIB_WLC = 0, 1
# fibrin nodes as immersed markers, or with their own velocity and the
# penalty coupling of the reference's fibrin FSI design
FIBCPL_MARKER, FIBCPL_PENALTY = 0, 1
MEM_SPRING, MEM_WALL, MEM_AREAVOL, MEM_BEND, MEM_ALL = 1, 2, 4, 8, 15
# the reference's disabled FEM bending chain, added to the chain it runs
MEM_FEMBEND = 16

P_NUMRECEPTORS, P_SEED, P_KSPRING, P_KF0, P_KR0, P_SHEAR, P_RHO0, P_L0, P_T0, P_M0, P_F0, \
    P_UMAX, P_NU, P_TAU, P_P0, P_CL, P_UNIT, P_KS, P_KV, P_KBEND = range(20)

_dp = C.POINTER(C.c_double)
_ip = C.POINTER(C.c_int)
_fp = C.POINTER(C.c_float)


class PfScene(C.Structure):
    _fields_ = [
        ("nx", C.c_int), ("ny", C.c_int), ("nz", C.c_int),
        ("dx", C.c_float), ("dt", C.c_float),
        ("params", C.c_float * 100),
        ("bc", C.c_int * 3), ("ibm_wrap", C.c_int * 3),
        ("body_force", C.c_double * 3),
        ("f_init", _dp), ("u_init", _dp), ("F_init", _dp), ("rho_init", _dp),
        ("n_platelets", C.c_int), ("n_elem", C.c_int), ("n_membrane", C.c_int),
        ("n_tri", C.c_int), ("n_node", C.c_int),
        ("tri", _ip), ("node_ntri", _ip), ("ring", _ip),
        ("spring_ptr", _ip), ("spring_nbr", _ip), ("spring_L0", _dp),
        ("S0", _dp), ("S0_all", _dp), ("V0", _dp),
        ("X", _dp), ("Y", _dp), ("RY", _dp), ("Z", _dp),
        ("membrane_forces", C.c_int),
        ("n_rec", C.c_int), ("rec_tri", _ip), ("rec_r1", _fp), ("rec_r2", _fp),
        ("rec_state", _ip), ("vwf", _ip),
        ("bond_model", C.c_int), ("p_on", C.c_double), ("p_off", C.c_double),
        ("morse", C.c_int), ("morse_intra", C.c_double * 4), ("morse_inter", C.c_double * 4),
        ("n_fib", C.c_int), ("fib_X", _dp), ("fib_Y", _dp), ("fib_Z", _dp),
        ("fib_fixed", _ip), ("fib_ptr", _ip), ("fib_nbr", _ip), ("fib_L0", _dp),
        ("fib_law", C.c_int), ("fib_k", C.c_double), ("fib_mass", C.c_double),
        ("seed", C.c_uint64), ("detach_rate", C.c_double),
        ("fib_coupling", C.c_int), ("fib_gamma", C.c_double), ("fib_node_mass", C.c_double),
        ("fib_kappa", C.c_double),
    ]


def _ptr(a, ctype):
    if a is None:
        return None
    return a.ctypes.data_as(C.POINTER(ctype))


def reference_params(*, dx: float, dt: float, nz: int, shear: float, rho0: float = 1.0239,
                     k_spring: float = 1e3, kr0: float = 3.21, receptors: float = 10688.0,
                     seed: float = 1018.0, mean_bond: float = 0.1, umax: float | None = None,
                     kf0: float | None = None, tau: float | None = None) -> np.ndarray:
    """Parameter table of gpuSEM_LB.c:1206-1233 (and the reader's fields of
    :148-344).  `umax`, `kf0`, `tau` override the derived values for
    workloads without a shear profile or with stressed bond rates."""
    p = np.zeros(100, dtype=np.float32)
    f32 = np.float32
    p[P_NUMRECEPTORS] = receptors
    p[P_SEED] = seed
    p[P_KSPRING] = k_spring
    p[P_KR0] = kr0
    p[P_SHEAR] = shear
    p[P_RHO0] = rho0
    dxf, dtf = f32(dx), f32(dt)
    U = float(p[P_SHEAR]) * (nz - 1) * float(dxf) if umax is None else float(umax)
    p[P_KF0] = 0.0165 * np.exp(0.00065 * float(p[P_SHEAR])) if kf0 is None else kf0
    rho = float(p[P_RHO0])
    L0 = 1.0
    p[P_L0] = L0
    p[P_T0] = L0 / U
    p[P_M0] = rho * L0 ** 3
    p[P_F0] = 1.0
    p[P_UMAX] = U
    p[P_NU] = 1.2e6 / rho
    if tau is None:
        p[P_TAU] = (3.0 * float(p[P_NU]) * float(dtf)) / float(dxf * dxf) + 0.5
    else:
        p[P_TAU] = tau
    p[P_P0] = rho * U * U
    p[P_CL] = float(f32(dxf / dtf)) / U
    p[P_UNIT] = 1e12
    kbt = 1.3806488e-8 * 300
    p[P_KS] = 600 * kbt / 2.0 / mean_bond / mean_bond
    p[P_KV] = 600 * kbt / 2.0 / mean_bond / mean_bond / mean_bond
    p[P_KBEND] = 500 * kbt * 1e-6
    return p


def lattice_C(params: np.ndarray, dx: float, dt: float) -> float:
    """Float-rounded lattice speed dx/dt/UMAX (LB_kernel.cu:1212)."""
    c = np.float32(np.float32(dx) / np.float32(dt))
    return float(np.float32(c / np.float32(params[P_UMAX])))


def force_to_lattice(params: np.ndarray, dx: float, dt: float) -> float:
    """Factor turning a reference-unit nodal force into a lattice-unit force
    density: F0/rho0/UMAX*1e12 * dt / C (LB_kernel.cu:1179,1296)."""
    f = np.float32(np.float32(params[P_F0]) / np.float32(params[P_RHO0]))
    f = np.float32(f / np.float32(params[P_UMAX]))
    f = np.float32(f * np.float32(params[P_UNIT]))
    return float(f) * float(np.float32(dt)) / lattice_C(params, dx, dt)


@dataclass
class Scene:
    nx: int
    ny: int
    nz: int
    dx: float
    dt: float
    params: np.ndarray
    bc: tuple = (BC_PERIODIC, BC_PERIODIC, BC_ZOUHE_SHEAR)
    ibm_wrap: tuple = (0, 1, 0)
    body_force: tuple = (0.0, 0.0, 0.0)
    f_init: np.ndarray | None = None
    u_init: np.ndarray | None = None
    F_init: np.ndarray | None = None
    rho_init: np.ndarray | None = None
    # platelets
    n_platelets: int = 0
    n_elem: int = 0
    n_membrane: int = 0
    tri: np.ndarray | None = None
    node_ntri: np.ndarray | None = None
    ring: np.ndarray | None = None
    spring_ptr: np.ndarray | None = None
    spring_nbr: np.ndarray | None = None
    spring_L0: np.ndarray | None = None
    S0: np.ndarray | None = None
    S0_all: np.ndarray | None = None
    V0: np.ndarray | None = None
    X: np.ndarray | None = None
    Y: np.ndarray | None = None
    RY: np.ndarray | None = None
    Z: np.ndarray | None = None
    membrane_forces: int = MEM_ALL
    # receptors
    n_rec: int = 0
    rec_tri: np.ndarray | None = None
    rec_r1: np.ndarray | None = None
    rec_r2: np.ndarray | None = None
    rec_state: np.ndarray | None = None
    vwf: np.ndarray | None = None
    bond_model: int = BOND_BELL
    p_on: float = 0.0
    p_off: float = 0.0
    # Morse
    morse: int = 0
    morse_intra: tuple = (1.0, 2.0, 0.3, 1.0)
    morse_inter: tuple = (1.0, 2.0, 0.3, 1.0)
    # fibrin
    n_fib: int = 0
    fib_X: np.ndarray | None = None
    fib_Y: np.ndarray | None = None
    fib_Z: np.ndarray | None = None
    fib_fixed: np.ndarray | None = None
    fib_ptr: np.ndarray | None = None
    fib_nbr: np.ndarray | None = None
    fib_L0: np.ndarray | None = None
    fib_law: int = FIB_HOOKE
    fib_k: float = 0.5
    fib_mass: float = 1.0
    seed: int = 1
    detach_rate: float = 0.0
    fib_coupling: int = FIBCPL_MARKER
    fib_gamma: float = 0.0
    fib_node_mass: float = 1.0
    fib_kappa: float = 1.0
    meta: dict = field(default_factory=dict)

    @property
    def n_nodes(self) -> int:
        return self.nx * self.ny * self.nz

    @property
    def n_tri(self) -> int:
        return 0 if self.tri is None else int(self.tri.shape[0])

    @property
    def n_node(self) -> int:
        return 0 if self.node_ntri is None else int(self.node_ntri.shape[0])

    def _arrays(self):
        def d(a):
            return None if a is None else np.ascontiguousarray(a, dtype=np.float64)

        def i(a):
            return None if a is None else np.ascontiguousarray(a, dtype=np.int32)

        def f(a):
            return None if a is None else np.ascontiguousarray(a, dtype=np.float32)

        return dict(
            f_init=d(self.f_init), u_init=d(self.u_init), F_init=d(self.F_init), rho_init=d(self.rho_init),
            tri=i(self.tri), node_ntri=i(self.node_ntri), ring=i(self.ring),
            spring_ptr=i(self.spring_ptr), spring_nbr=i(self.spring_nbr), spring_L0=d(self.spring_L0),
            S0=d(self.S0), S0_all=d(self.S0_all), V0=d(self.V0),
            X=d(self.X), Y=d(self.Y), RY=d(self.RY), Z=d(self.Z),
            rec_tri=i(self.rec_tri), rec_r1=f(self.rec_r1), rec_r2=f(self.rec_r2),
            rec_state=i(self.rec_state), vwf=i(self.vwf),
            fib_X=d(self.fib_X), fib_Y=d(self.fib_Y), fib_Z=d(self.fib_Z), fib_fixed=i(self.fib_fixed),
            fib_ptr=i(self.fib_ptr), fib_nbr=i(self.fib_nbr), fib_L0=d(self.fib_L0),
        )

    def to_c(self) -> PfScene:
        """ctypes view of the scene; the returned struct keeps its arrays alive."""
        a = self._arrays()
        s = PfScene()
        s.nx, s.ny, s.nz = self.nx, self.ny, self.nz
        s.dx, s.dt = self.dx, self.dt
        s.params[:] = [float(v) for v in np.asarray(self.params, dtype=np.float32)]
        s.bc[:] = list(self.bc)
        s.ibm_wrap[:] = list(self.ibm_wrap)
        s.body_force[:] = list(self.body_force)
        s.f_init, s.u_init, s.F_init = _ptr(a["f_init"], C.c_double), _ptr(a["u_init"], C.c_double), \
            _ptr(a["F_init"], C.c_double)
        s.rho_init = _ptr(a["rho_init"], C.c_double)
        s.n_platelets, s.n_elem, s.n_membrane = self.n_platelets, self.n_elem, self.n_membrane
        s.n_tri, s.n_node = self.n_tri, self.n_node
        for k in ("tri", "node_ntri", "ring", "spring_ptr", "spring_nbr", "rec_tri", "rec_state", "vwf",
                  "fib_fixed", "fib_ptr", "fib_nbr"):
            setattr(s, k, _ptr(a[k], C.c_int))
        for k in ("spring_L0", "S0", "S0_all", "V0", "X", "Y", "RY", "Z", "fib_X", "fib_Y", "fib_Z",
                  "fib_L0"):
            setattr(s, k, _ptr(a[k], C.c_double))
        s.rec_r1, s.rec_r2 = _ptr(a["rec_r1"], C.c_float), _ptr(a["rec_r2"], C.c_float)
        s.membrane_forces = self.membrane_forces
        s.n_rec = self.n_rec
        s.bond_model, s.p_on, s.p_off = self.bond_model, self.p_on, self.p_off
        s.morse = self.morse
        s.morse_intra[:] = list(self.morse_intra)
        s.morse_inter[:] = list(self.morse_inter)
        s.n_fib = self.n_fib
        s.fib_law, s.fib_k, s.fib_mass = self.fib_law, self.fib_k, self.fib_mass
        s.seed = int(self.seed) & ((1 << 64) - 1)
        s.detach_rate = self.detach_rate
        s.fib_coupling, s.fib_gamma = self.fib_coupling, self.fib_gamma
        s.fib_node_mass, s.fib_kappa = self.fib_node_mass, self.fib_kappa
        s._keep = a  # noqa: SLF001 -- keeps the arrays referenced by the pointers alive
        return s


_ARRAY_FIELDS = ("params", "f_init", "u_init", "F_init", "rho_init", "tri", "node_ntri", "ring", "spring_ptr", "spring_nbr",
                 "spring_L0", "S0", "S0_all", "V0", "X", "Y", "RY", "Z", "rec_tri", "rec_r1", "rec_r2",
                 "rec_state", "vwf", "fib_X", "fib_Y", "fib_Z", "fib_fixed", "fib_ptr", "fib_nbr", "fib_L0")
_SCALAR_FIELDS = ("nx", "ny", "nz", "dx", "dt", "bc", "ibm_wrap", "body_force", "n_platelets", "n_elem",
                  "n_membrane", "membrane_forces", "n_rec", "bond_model", "p_on", "p_off", "morse",
                  "morse_intra", "morse_inter", "n_fib", "fib_law", "fib_k", "fib_mass", "seed", "detach_rate",
                  "fib_coupling", "fib_gamma", "fib_node_mass", "fib_kappa")


def scene_to_dict(sc: Scene, prefix: str = "scene.") -> dict:
    """Flat dict of arrays (for np.savez) that `scene_from_dict` inverts."""
    out = {}
    for k in _ARRAY_FIELDS:
        v = getattr(sc, k)
        if v is not None:
            out[prefix + k] = np.asarray(v)
    for k in _SCALAR_FIELDS:
        out[prefix + k] = np.asarray(getattr(sc, k))
    return out


def scene_from_dict(d, prefix: str = "scene.") -> Scene:
    kw = {}
    for k in _SCALAR_FIELDS:
        if (prefix + k) not in d:
            continue  # written before the field existed: the default
        v = np.asarray(d[prefix + k])
        kw[k] = tuple(v.tolist()) if v.ndim else v.item()
    for k in _ARRAY_FIELDS:
        kw[k] = np.asarray(d[prefix + k]) if (prefix + k) in d else None
    return Scene(**kw)
