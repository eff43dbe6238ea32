"""CPU oracle for the noFluidX3D tetra-mesh step — TEST INFRASTRUCTURE ONLY.

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg import this package, and
only as the checker (or, for bench.py, as the timed CPU baseline). The product package
nofluidx3d_gb300 never imports it and has no CPU fallback.

Two libraries:
  * libnfx_oracle.so — the C restatement in nfx_oracle.c / oracle_body.h (FP64 as the
    reference ships, plus an FP32 variant, serial and OpenMP), built by build();
  * oracle/_ref/libnfxref.so — the reference's own kernels compiled through a shim
    (build_ref.py), present only where the reference tree is; used to pin the restatement
    and to generate tests/golden/.

Array layouts are the reference's: points/velocities/forces SoA (3*Np), tets SoA (4*Nt),
edge vectors SoA (9*Nt). See nfx_oracle.c.
"""

from __future__ import annotations

import ctypes as C
import os
import subprocess
from dataclasses import dataclass, field
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
BUILD_DIR = HERE / "_build"
LIB_PATH = BUILD_DIR / "libnfx_oracle.so"
REF_LIB_PATH = HERE / "_ref" / "libnfxref.so"

MODEL_MR, MODEL_SVK, MODEL_SVKK, MODEL_VP = 0, 1, 2, 3
SUBSTRATE, PLANE, SPHERE = 0, 1, 2
SPHERE_INTEGRAL = 3  # InteractionSphereIntegral.cl
INTEGRATOR_VV, INTEGRATOR_VV2 = 0, 1  # VelocityVerlet.cl (unit mass), velocityVerlet2.cl (lumped masses)


def build(force: bool = False) -> Path:
    """Compile nfx_oracle.c for this host (x86-64 here, aarch64 on the GPU machine)."""
    src = [HERE / "nfx_oracle.c", HERE / "oracle_body.h"]
    if not force and LIB_PATH.exists() and all(LIB_PATH.stat().st_mtime >= s.stat().st_mtime for s in src):
        return LIB_PATH
    BUILD_DIR.mkdir(exist_ok=True)
    tmp = LIB_PATH.with_suffix(f".{os.getpid()}.tmp")
    cmd = ["gcc", "-O2", "-fPIC", "-shared", "-fopenmp", "-ffp-contract=off",
           str(HERE / "nfx_oracle.c"), "-lm", "-o", str(tmp)]
    subprocess.run(cmd, check=True)
    os.replace(tmp, LIB_PATH)
    return LIB_PATH


class _Contact(C.Structure):
    _fields_ = [("kind", C.c_int), ("k", C.c_double), ("radius", C.c_double),
                ("p0", C.c_double), ("v", C.c_double), ("tmove", C.c_double)]


class _Problem(C.Structure):
    _fields_ = [("np", C.c_long), ("nt", C.c_long), ("tets", C.c_void_p), ("edge", C.c_void_p),
                ("vol", C.c_void_p), ("model", C.c_int), ("E", C.c_double), ("nu", C.c_double),
                ("mr", C.c_double), ("n_contacts", C.c_int), ("contacts", _Contact * 4),
                ("xi", C.c_double), ("fix_top_bottom", C.c_int), ("record_contact", C.c_int),
                ("integrator", C.c_int), ("masses", C.c_void_p)]


class _State(C.Structure):
    _fields_ = [(n, C.c_void_p) for n in
                ("points", "vel", "force", "fold", "acc", "Fp", "vonMises", "pressure", "vp_par")]


_lib = None


def lib():
    global _lib
    if _lib is None:
        _lib = C.CDLL(str(build()))
        for sfx in ("_f64", "_f32"):
            f = getattr(_lib, "ora_run" + sfx)
            f.restype = C.c_long
            f.argtypes = [C.POINTER(_Problem), C.POINTER(_State), C.c_long, C.c_long, C.c_long,
                          C.c_void_p, C.c_long]
            f = getattr(_lib, "ora_run_par" + sfx)
            f.restype = C.c_long
            f.argtypes = [C.POINTER(_Problem), C.POINTER(_State), C.c_long, C.c_long, C.c_int]
            f = getattr(_lib, "ora_readout" + sfx)
            f.restype = C.c_double
            f.argtypes = [C.POINTER(_Problem), C.POINTER(_State), C.c_long]
            f = getattr(_lib, "ora_tet_force" + sfx)
            f.restype = None
        _lib.ora_max_threads.restype = C.c_int
    return _lib


def _ptr(a: np.ndarray | None) -> int | None:
    return None if a is None else a.ctypes.data


@dataclass
class Contact:
    """kind: SUBSTRATE / PLANE / SPHERE; position(t) = p0 - v*min(t, tmove)."""

    kind: int
    k: float = 0.1
    p0: float = 0.0
    v: float = 0.0
    tmove: float = 1e300
    radius: float = 0.0

    def position(self, t: float) -> float:
        if self.kind == SUBSTRATE:
            return self.p0
        return self.p0 - self.v * t if t <= self.tmove else self.p0 - self.v * self.tmove


@dataclass
class Problem:
    """A cell problem in the reference's layouts. points (Np,3), tets (Nt,4)."""

    points: np.ndarray
    tets: np.ndarray
    model: int = MODEL_MR
    E: float = 1.0
    nu: float = 0.3
    mr: float = 1.0
    vp_par: tuple = (0.0,) * 8  # mu1, mu2, kappa, flowExp, yield, flowRate, hardThr, hardExp
    contacts: list = field(default_factory=list)
    xi: float = 0.005
    fix_top_bottom: bool = False
    record_contact: int = -1
    integrator: int = INTEGRATOR_VV
    density: float = 1.0  # lumped masses of INTEGRATOR_VV2

    @property
    def np_(self) -> int:
        return int(self.points.shape[0])

    @property
    def nt(self) -> int:
        return int(self.tets.shape[0])

    def edge_base(self) -> int:
        return 3 if self.model == MODEL_VP else 0


def lumped_masses(points: np.ndarray, tets: np.ndarray, density: float = 1.0) -> np.ndarray:
    """Nodal masses of VelocityVerlet2, nofluidx3d/SimulationLegacy.py:911-924: every tetra adds a
    quarter of density * V0 (TetraCell volumes, TetraCell.py:39-41) to each of its corners, in tetra
    order then corner order, as the reference's Python loop does."""
    from nofluidx3d_gb300.mesh import signed_volumes  # setup math only

    q = 0.25 * density * signed_volumes(points, tets)
    m = np.zeros(points.shape[0])
    np.add.at(m, np.asarray(tets, np.int64).reshape(-1), np.repeat(q, 4))
    return m


class State:
    """Mutable simulation state for one precision ('f64' or 'f32')."""

    def __init__(self, prob: Problem, precision: str = "f64"):
        from nofluidx3d_gb300.mesh import edge_vectors, signed_volumes  # setup math only

        dt = np.float64 if precision == "f64" else np.float32
        self.precision = precision
        self.dtype = dt
        self.prob = prob
        npn, nt = prob.np_, prob.nt
        self.points = np.ascontiguousarray(prob.points.T.reshape(-1), dtype=dt)  # SoA (Fortran)
        self.vel = np.zeros(3 * npn, dt)
        self.force = np.zeros(3 * npn, dt)
        self.fold = np.zeros(3 * npn, dt)
        self.tets = np.ascontiguousarray(prob.tets.T.reshape(-1), dtype=np.uint32)
        ev = edge_vectors(prob.points, prob.tets, base=prob.edge_base())
        self.edge = np.ascontiguousarray(ev.T.reshape(-1), dtype=dt)
        self.vol = np.ascontiguousarray(signed_volumes(prob.points, prob.tets), dtype=dt)
        self.acc = np.zeros(nt, dt)
        self.Fp = np.ascontiguousarray(np.repeat(np.eye(3).reshape(9), nt), dtype=dt)
        self.vonMises = np.zeros(nt, dt)
        self.pressure = np.zeros(nt, dt)
        self.vp_par = np.array(prob.vp_par, dt)
        self.time = 0
        self._cprob = _Problem()
        p = self._cprob
        p.np, p.nt = npn, nt
        p.tets, p.edge, p.vol = _ptr(self.tets), _ptr(self.edge), _ptr(self.vol)
        p.model, p.E, p.nu, p.mr = prob.model, prob.E, prob.nu, prob.mr
        p.n_contacts = len(prob.contacts)
        if p.n_contacts > 4:
            raise ValueError("at most 4 contacts")
        for i, c in enumerate(prob.contacts):
            p.contacts[i] = _Contact(c.kind, c.k, c.radius, c.p0, c.v, min(c.tmove, 1e300))
        p.xi, p.fix_top_bottom, p.record_contact = prob.xi, int(prob.fix_top_bottom), prob.record_contact
        self.masses = np.ascontiguousarray(lumped_masses(prob.points, prob.tets, prob.density), dtype=dt)
        p.integrator, p.masses = int(prob.integrator), _ptr(self.masses)
        self._cstate = _State(*[_ptr(a) for a in (self.points, self.vel, self.force, self.fold, self.acc,
                                                  self.Fp, self.vonMises, self.pressure, self.vp_par)])

    def positions(self) -> np.ndarray:
        return self.points.reshape(3, -1).T.astype(np.float64)

    def velocities(self) -> np.ndarray:
        return self.vel.reshape(3, -1).T.astype(np.float64)

    def run(self, nsteps: int, record_every: int = 0, parallel: bool = False, threads: int = 0):
        """Advance nsteps. Returns the curve rows (t, indentation, force) when recording."""
        L = lib()
        sfx = "_" + self.precision
        if parallel:
            getattr(L, "ora_run_par" + sfx)(C.byref(self._cprob), C.byref(self._cstate), self.time,
                                             nsteps, threads)
            self.time += nsteps
            return None
        rows = (nsteps // record_every + 1) if record_every > 0 else 0
        curve = np.zeros((max(rows, 1), 3), np.float64)
        n = getattr(L, "ora_run" + sfx)(C.byref(self._cprob), C.byref(self._cstate), self.time, nsteps,
                                         record_every, _ptr(curve) if rows else None, rows)
        self.time += nsteps
        return curve[:n] if rows else None

    def readout(self) -> float:
        """Indenter force of the recorded contact at the current time (lattice units)."""
        f = getattr(lib(), "ora_readout_" + self.precision)
        return float(f(C.byref(self._cprob), C.byref(self._cstate), self.time))


def max_threads() -> int:
    return int(lib().ora_max_threads())


# ----------------------------------------------------------------------------------------------
# The reference's own kernels (oracle/_ref), driven like Simulation.timeStep (Simulation.py:232-237)
# ----------------------------------------------------------------------------------------------
_ref = None


def ref_available() -> bool:
    return REF_LIB_PATH.exists()


def ref_lib():
    global _ref
    if _ref is None:
        if not REF_LIB_PATH.exists():
            raise FileNotFoundError(f"{REF_LIB_PATH} not built (python oracle/build_ref.py)")
        _ref = C.CDLL(str(REF_LIB_PATH))
        v, d, L, I = C.c_void_p, C.c_double, C.c_long, C.c_int
        _ref.ref_tetra.argtypes = [v, v, v, v, v, L, L, I, d, d, d]
        _ref.ref_vp.argtypes = [v, v, v, v, v, L, L, v, v, v, v, v]
        _ref.ref_substrate.argtypes = [v, v, L, d, d]
        _ref.ref_plane.argtypes = [v, v, L, d, d]
        _ref.ref_sphere.argtypes = [v, v, L, d, d, d]
        _ref.ref_vv.argtypes = [v, v, v, v, L, d, I]
        _ref.ref_vv2.argtypes = [v, v, v, v, v, L, d]
        _ref.ref_sphere_integral.argtypes = [v, v, v, L, L, d, d, d]
        for f in (_ref.ref_tetra, _ref.ref_vp, _ref.ref_substrate, _ref.ref_plane, _ref.ref_sphere, _ref.ref_vv,
                  _ref.ref_vv2, _ref.ref_sphere_integral):
            f.restype = None
    return _ref


def ref_run(st: State, nsteps: int, record_every: int = 0):
    """Advance an f64 State with the reference kernels; curve rows as State.run."""
    assert st.precision == "f64"
    R = ref_lib()
    P = st.prob
    npn, nt = P.np_, P.nt
    tets_i32 = st.tets.view(np.int32)
    rows = []

    def record(t):
        rows.append((float(t), 0.0, st.readout()))
        if 0 <= P.record_contact < len(P.contacts):
            c = P.contacts[P.record_contact]
            rows[-1] = (float(t), c.position(0) - c.position(t), rows[-1][2])

    if record_every > 0:
        record(st.time)
    for s in range(nsteps):
        t = st.time
        if P.model == MODEL_VP:
            R.ref_vp(_ptr(st.force), _ptr(st.points), _ptr(st.tets), _ptr(st.edge), _ptr(st.vol), npn, nt,
                     _ptr(st.vp_par), _ptr(st.acc), _ptr(st.Fp), _ptr(st.vonMises), _ptr(st.pressure))
        else:
            R.ref_tetra(_ptr(st.force), _ptr(st.points), _ptr(tets_i32), _ptr(st.edge), _ptr(st.vol), npn, nt,
                        P.model, P.E, P.nu, P.mr)
        for c in P.contacts:
            pos = c.position(t)
            if c.kind == SUBSTRATE:
                R.ref_substrate(_ptr(st.force), _ptr(st.points), npn, pos, c.k)
            elif c.kind == PLANE:
                R.ref_plane(_ptr(st.force), _ptr(st.points), npn, pos, c.k)
            elif c.kind == SPHERE_INTEGRAL:
                R.ref_sphere_integral(_ptr(st.force), _ptr(st.points), _ptr(st.tets), npn, nt, c.radius, pos, c.k)
            else:
                R.ref_sphere(_ptr(st.force), _ptr(st.points), npn, c.radius, pos, c.k)
        if P.integrator == INTEGRATOR_VV2:
            R.ref_vv2(_ptr(st.points), _ptr(st.vel), _ptr(st.force), _ptr(st.fold), _ptr(st.masses), npn, P.xi)
        else:
            R.ref_vv(_ptr(st.points), _ptr(st.vel), _ptr(st.force), _ptr(st.fold), npn, P.xi,
                     int(P.fix_top_bottom))
        st.time += 1
        if record_every > 0 and (s + 1) % record_every == 0:
            record(st.time)
    return np.array(rows) if record_every > 0 else None
