"""Learned surrogate of the indentation experiment and surrogate-assisted inverse fitting.

A cell of fixed radius R (Kuhn sphere, Mooney-Rivlin + viscoplastic, the step of this package)
is indented by a sphere at constant speed to 30 % of R; its force-depth curve, sampled at 64
depths, depends on six inputs: shear modulus mu, Mooney-Rivlin fraction r = mu1 / mu (mu1 =
r mu, mu2 = (1 - r) mu), bulk/shear ratio K / mu, yield stress Y, plastic viscosity eta
(power-law flow with exponent 1, rate Y / eta, as workloads.Workload maps it) and the indenter
radius Rs. The surrogate (mlp.MLP, 6 -> 256 x 3 -> 64, trained on the GPU by the package's own
kernels) maps the inputs, scaled to [-1, 1], to the curve divided by the constant 1e-3 R^2 (the
middle of the shear-modulus range times R^2), trained on the squared relative curve error. Its
output carries the gain exp(a u_mu) = mu / 1e-3 (nfx_mlp_set_output_gain on the shear-modulus
input), so the layers learn the curve per unit shear modulus, which varies far less across the
box than the curve itself, while fitting the inputs still follows exact gradients of the curve.

Inverse fit: given a measured curve and the known indenter radius, find the five material
inputs. The plain method is a batched Levenberg-Marquardt on the simulator (finite-difference
Jacobians, every evaluation a full simulation). The surrogate-assisted method proposes inputs by
gradient descent through the network (many starts per target, no simulation), has the simulator
verify each proposal, and refines it by defect correction (output space mapping): the target is
shifted by the simulator-minus-network difference at the current point and the network's inputs
are refitted to the shifted target, one verifying simulation per iteration, for as long as the
simulated error keeps improving. Every reported error is measured against the simulator.

The reference has no learned part; curves come from the batched simulator (core.Batch), whose
cells evolve bit for bit as the plain path (core.CellSim) runs them alone.
"""

from __future__ import annotations

import math
import time
from dataclasses import dataclass, field

import numpy as np

from .core import Batch
from .mesh import kuhn_sphere
from .workloads import Workload

PARAM_NAMES = ("shear_modulus", "mr_fraction", "bulk_ratio", "yield_stress", "viscosity", "indenter_radius")
# (low, high, log scale); the indenter radius range is relative to the cell radius
_RANGES = (
    (2e-4, 5e-3, True),
    (0.5, 1.0, False),
    (5.0, 50.0, True),
    (5e-5, 1e-3, True),
    (1e-2, 1e-1, True),
    (0.25, 1.5, True),
)
N_IN = 6
FREE_MATERIAL = np.array([True, True, True, True, True, False])  # the indenter radius is known


@dataclass(frozen=True)
class Protocol:
    """The indentation experiment every curve comes from."""

    radius: float = 16.0
    speed: float = 1e-4          # indenter descent per step (the indentation speed of the workloads)
    depth_frac: float = 0.3      # curves span depths 0 .. depth_frac * radius
    n_depths: int = 64
    record_every: int = 100
    xi: float = 1e-2             # velocity damping
    k: float = 0.1               # contact penalty
    jitter: float = 0.02
    mesh_seed: int = 0
    tile_tets: int = 128         # batch tile size (0: autotune)
    max_cells: int = 2048        # cells per batch launch
    # Curves rougher than this (norm of second differences over the curve's norm; smooth curves
    # sit near 0.02) come from cells at the explicit scheme's stability limit (stiff materials at
    # dt = 1 with unit nodal mass, which the FP64 reference scheme cannot run either) and are
    # discarded like cells that raised a status.
    max_roughness: float = 0.1

    @property
    def max_depth(self) -> float:
        return self.depth_frac * self.radius

    @property
    def steps(self) -> int:
        n = int(math.ceil(self.max_depth / self.speed / self.record_every - 1e-9))
        return n * self.record_every

    def depths(self) -> np.ndarray:
        return np.linspace(0.0, self.max_depth, self.n_depths)

    def bounds(self) -> tuple[np.ndarray, np.ndarray]:
        lo = np.array([r[0] for r in _RANGES])
        hi = np.array([r[1] for r in _RANGES])
        lo[5] *= self.radius
        hi[5] *= self.radius
        return lo, hi

    def mesh(self):
        return kuhn_sphere(self.radius, self.jitter, self.mesh_seed)


def to_unit(params: np.ndarray, proto: Protocol) -> np.ndarray:
    """Physical inputs [n, 6] -> [-1, 1] (log scale where the range is)."""
    p = np.asarray(params, np.float64).reshape(-1, N_IN)
    lo, hi = proto.bounds()
    u = np.empty_like(p)
    for j, (_, _, lg) in enumerate(_RANGES):
        a, b, x = (np.log(lo[j]), np.log(hi[j]), np.log(p[:, j])) if lg else (lo[j], hi[j], p[:, j])
        u[:, j] = 2.0 * (x - a) / (b - a) - 1.0
    return u


def from_unit(u: np.ndarray, proto: Protocol) -> np.ndarray:
    u = np.clip(np.asarray(u, np.float64).reshape(-1, N_IN), -1.0, 1.0)
    lo, hi = proto.bounds()
    p = np.empty_like(u)
    for j, (_, _, lg) in enumerate(_RANGES):
        if lg:
            a, b = np.log(lo[j]), np.log(hi[j])
            p[:, j] = np.exp(a + (u[:, j] + 1.0) * 0.5 * (b - a))
        else:
            p[:, j] = lo[j] + (u[:, j] + 1.0) * 0.5 * (hi[j] - lo[j])
    return p


def sample_params(n: int, proto: Protocol, seed: int = 0) -> np.ndarray:
    """n input sets drawn uniformly in the unit box (log-uniform where the range is log)."""
    rng = np.random.default_rng(seed)
    return from_unit(rng.uniform(-1.0, 1.0, (n, N_IN)), proto)


def workload(p: np.ndarray, proto: Protocol) -> Workload:
    mu, r, kr, Y, eta, Rs = (float(v) for v in p)
    return Workload("surrogate cell", radius=proto.radius, material="mr_vp", C10=r * mu / 2.0,
                    C01=(1.0 - r) * mu / 2.0, K=kr * mu, yield_stress=Y, viscosity=eta, indenter="sphere",
                    sphere_radius=Rs, speed=proto.speed, d0=None, k=proto.k, xi=proto.xi, steps=proto.steps,
                    record_every=proto.record_every, jitter=proto.jitter, seed=proto.mesh_seed)


def force_scale(proto: Protocol) -> float:
    """Curves are learned as force / (1e-3 R^2): a constant, so that fitting the network's inputs
    to a measured curve is a plain gradient descent."""
    return 1e-3 * proto.radius ** 2


@dataclass
class SimStats:
    """Full simulations run and the wall time they took."""

    sims: int = 0
    seconds: float = 0.0
    tetra_steps: float = 0.0


def simulate_curves(params: np.ndarray, proto: Protocol, stats: SimStats | None = None) -> np.ndarray:
    """Force at proto.depths() for every input row (one full simulation each, batched on the
    GPU in launches of proto.max_cells cells sharing one mesh). Rows whose simulation raised a
    status (an inverted tetra, a non-finite value) or whose curve is rougher than
    proto.max_roughness come back as NaN."""
    P = np.asarray(params, np.float64).reshape(-1, N_IN)
    mesh = proto.mesh()
    depths = proto.depths()
    rows = proto.steps // proto.record_every + 1
    out = np.full((P.shape[0], proto.n_depths), np.nan)
    t0 = time.perf_counter()
    for a in range(0, P.shape[0], proto.max_cells):
        chunk = P[a:a + proto.max_cells]
        b = Batch(0, tile_tets=proto.tile_tets)
        try:
            first = None
            for p in chunk:
                c = workload(p, proto).add_to_batch(b, mesh, like=first)
                first = c if first is None else first
            b.set_record(1, proto.record_every, rows)
            b.finalize()
            b.step(proto.steps)
            b.record_now()
            bad = b.cell_status() != 0
            for i in range(chunk.shape[0]):
                cv = b.curve(i)
                ind, force = cv[:, 1], cv[:, 2]
                if not bad[i] and cv.shape[0] == rows and np.all(np.isfinite(force)):
                    c = np.interp(depths, ind, force)
                    if roughness(c) <= proto.max_roughness:
                        out[a + i] = c
        finally:
            b.close()
    if stats is not None:
        stats.sims += P.shape[0]
        stats.seconds += time.perf_counter() - t0
        stats.tetra_steps += float(P.shape[0]) * mesh.num_tetra * proto.steps
    return out


def roughness(curve: np.ndarray) -> float:
    """Norm of the second differences of a curve over its norm."""
    c = np.asarray(curve, np.float64)
    return float(np.linalg.norm(np.diff(c, 2)) / max(np.linalg.norm(c), 1e-300))


def curve_error(curves: np.ndarray, targets: np.ndarray) -> np.ndarray:
    """Relative L2 error of each curve against its target."""
    c = np.asarray(curves, np.float64)
    t = np.asarray(targets, np.float64)
    return np.linalg.norm(c - t, axis=-1) / np.maximum(np.linalg.norm(t, axis=-1), 1e-300)


class Surrogate:
    """The MLP surrogate of one Protocol: inputs in [-1, 1], outputs curve / force_scale."""

    def __init__(self, proto: Protocol, width: int = 256, depth: int = 3, max_batch: int = 1024, device: int = 0,
                 seed: int = 0):
        from .mlp import MLP

        self.proto = proto
        self.net = MLP(N_IN, width, depth, proto.n_depths, max_batch=max_batch, device=device)
        self.net.set_params(_he_init(N_IN, width, depth, proto.n_depths, seed))
        lo, hi = proto.bounds()
        # u_mu in [-1, 1] spans log(mu) over [lo, hi]: exp(a u_mu) = mu / sqrt(lo hi) = mu / 1e-3
        self.net.set_output_gain(0, 0.5 * math.log(hi[0] / lo[0]))
        self.history: np.ndarray | None = None

    def close(self) -> None:
        self.net.close()

    def _xy(self, params, curves):
        x = to_unit(params, self.proto).astype(np.float32)
        y = (np.asarray(curves, np.float64) / force_scale(self.proto)).astype(np.float32)
        return x, y

    def train(self, params: np.ndarray, curves: np.ndarray, steps: int = 20000, batch: int = 512,
              lr: float = 2e-3, lr_min: float = 1e-5, weight_decay: float = 1e-5, seed: int = 0) -> np.ndarray:
        """AdamW on the squared relative curve error (each row weighted by 1 / ||y||^2)."""
        ok = np.all(np.isfinite(curves), axis=1)
        x, y = self._xy(params[ok], curves[ok])
        w = (1.0 / np.maximum((y.astype(np.float64) ** 2).sum(1), 1e-30)).astype(np.float32)
        self.history = self.net.train(x, y, steps=steps, batch=min(batch, x.shape[0]), lr=lr, lr_min=lr_min,
                                      weight_decay=weight_decay, weight=w, seed=seed)
        return self.history

    def predict(self, params: np.ndarray) -> np.ndarray:
        P = np.asarray(params, np.float64).reshape(-1, N_IN)
        y = self.net.forward(to_unit(P, self.proto).astype(np.float32)).astype(np.float64)
        return y * force_scale(self.proto)

    def propose(self, targets: np.ndarray, indenter_radius: np.ndarray, starts: int = 16, steps: int = 400,
                lr: float = 2e-2, seed: int = 0) -> np.ndarray:
        """Material inputs whose predicted curves best match the targets (known indenter radius):
        Adam on the network's inputs from `starts` starting points per target (batched in one
        call per chunk), then the start with the lowest relative error wins. No simulation."""
        T = np.asarray(targets, np.float64).reshape(-1, self.proto.n_depths)
        Rs = np.asarray(indenter_radius, np.float64).reshape(-1)
        n = T.shape[0]
        rng = np.random.default_rng(seed)
        u0 = rng.uniform(-0.9, 0.9, (n, starts, N_IN))
        u0[:, 0, :5] = 0.0  # the centre of the box is always one start
        lo_u, hi_u = -np.ones(N_IN, np.float32), np.ones(N_IN, np.float32)
        known = from_unit(np.zeros((n, N_IN)), self.proto)
        known[:, 5] = Rs
        u0[:, :, 5] = to_unit(known, self.proto)[:, 5][:, None]
        y_all = (T / force_scale(self.proto)).astype(np.float32)
        w_all = (1.0 / np.maximum((y_all.astype(np.float64) ** 2).sum(1), 1e-30)).astype(np.float32)
        flat_u = u0.reshape(-1, N_IN)
        flat_y = np.repeat(y_all, starts, axis=0)
        flat_w = np.repeat(w_all, starts)
        flat_t = np.repeat(T, starts, axis=0)
        rows = self.net.max_batch
        for a in range(0, flat_u.shape[0], rows):
            u, _ = self.net.fit_inputs(flat_u[a:a + rows].astype(np.float32), flat_y[a:a + rows], FREE_MATERIAL,
                                       lo_u, hi_u, steps=steps, lr=lr, weight=flat_w[a:a + rows])
            flat_u[a:a + rows] = u
        P = from_unit(flat_u, self.proto)
        err = curve_error(self.predict(P), flat_t).reshape(n, starts)
        k = np.argmin(err, axis=1)
        best_u = flat_u.reshape(n, starts, N_IN)[np.arange(n), k]
        out = from_unit(best_u, self.proto)
        out[:, 5] = Rs  # exactly the known radius (the unit coordinate went through float32)
        return out


def _he_init(n_in: int, width: int, depth: int, n_out: int, seed: int) -> np.ndarray:
    rng = np.random.default_rng(seed)
    dims = [n_in] + [width] * depth + [n_out]
    parts = []
    for i in range(len(dims) - 1):
        lim = math.sqrt(6.0 / dims[i])
        parts.append(rng.uniform(-lim, lim, dims[i + 1] * dims[i]))
        parts.append(np.zeros(dims[i + 1]))
    return np.concatenate(parts).astype(np.float32)


@dataclass
class FitResult:
    params: np.ndarray            # [n, 6] fitted inputs (indenter radius as given)
    curves: np.ndarray            # [n, n_depths] simulated curves at the fitted inputs
    error: np.ndarray             # [n] relative L2 error against the targets
    sims: np.ndarray              # [n] full simulations spent on each target
    iterations: np.ndarray        # [n] Levenberg-Marquardt iterations run
    seconds: float = 0.0          # wall time (simulations, network calls and host work)


def lm_fit(targets: np.ndarray, start: np.ndarray, proto: Protocol, max_iter: int = 30, h: float = 0.02,
           lam0: float = 1e-2, rtol: float = 1e-3, start_curves: np.ndarray | None = None,
           stats: SimStats | None = None, simulate=None) -> FitResult:
    """Batched Levenberg-Marquardt on the simulator over the five material inputs in unit
    coordinates (the indenter radius stays as in `start`). Each iteration of each active target
    costs 5 simulations for a forward-difference Jacobian and 1 for the trial point; a target
    stops when an accepted step improves its error by less than rtol relative, or after four
    rejected steps in a row (the damping grows 4x per rejection). start_curves (simulated curves at `start`, if already known) saves
    the first evaluation. simulate(params, proto, stats) -> curves defaults to simulate_curves."""
    sim = simulate if simulate is not None else simulate_curves
    t0 = time.perf_counter()
    T = np.asarray(targets, np.float64).reshape(-1, proto.n_depths)
    n = T.shape[0]
    tn = np.maximum(np.linalg.norm(T, axis=1), 1e-300)
    u = to_unit(start, proto)
    radius = np.asarray(start, np.float64).reshape(-1, N_IN)[:, 5].copy()

    def phys(uu, rows):  # unit -> physical with the known indenter radius kept exact
        q = from_unit(uu, proto)
        q[:, 5] = radius[rows]
        return q

    sims = np.zeros(n, np.int64)
    its = np.zeros(n, np.int64)
    if start_curves is None:
        F = sim(phys(u, np.arange(n)), proto, stats)
        sims += 1
    else:
        F = np.asarray(start_curves, np.float64).copy()
    e = curve_error(F, T)
    e[~np.isfinite(e)] = np.inf
    lam = np.full(n, lam0)
    active = np.isfinite(e)
    rejects = np.zeros(n, np.int64)
    free = np.flatnonzero(FREE_MATERIAL)
    for _ in range(max_iter):
        idx = np.flatnonzero(active)
        if idx.size == 0:
            break
        m = idx.size
        steps = np.where(u[idx][:, free] + h <= 1.0, h, -h)          # [m, 5]
        U = np.repeat(u[idx][None], free.size, axis=0)               # [5, m, 6]
        for q, j in enumerate(free):
            U[q, :, j] += steps[:, q]
        FJ = sim(phys(U.reshape(-1, N_IN), np.tile(idx, free.size)), proto, stats).reshape(free.size, m, -1)
        J = (FJ - F[idx][None]) / steps.T[:, :, None] / tn[idx][None, :, None]   # [5, m, nd]
        J = np.nan_to_num(np.transpose(J, (1, 2, 0)))                # [m, nd, 5]
        r = (F[idx] - T[idx]) / tn[idx][:, None]                     # [m, nd]
        A = np.einsum("mdi,mdj->mij", J, J)
        g = np.einsum("mdi,md->mi", J, r)
        D = np.einsum("mii->mi", A)
        # Marquardt scaling plus a small ridge, so directions the curve does not see stay solvable
        ridge = 1e-10 * np.maximum(D.max(axis=1), 1e-30)
        A = A + np.einsum("mi,ij->mij", lam[idx][:, None] * D + ridge[:, None], np.eye(free.size))
        delta = -np.linalg.solve(A, g[..., None])[..., 0]
        delta = np.clip(delta, -0.5, 0.5)
        un = u[idx].copy()
        un[:, free] = np.clip(un[:, free] + delta, -1.0, 1.0)
        Fn = sim(phys(un, idx), proto, stats)
        en = curve_error(Fn, T[idx])
        en[~np.isfinite(en)] = np.inf
        sims[idx] += free.size + 1
        its[idx] += 1
        better = en < e[idx]
        gain = np.where(better, (e[idx] - en) / np.maximum(e[idx], 1e-300), 0.0)
        acc = idx[better]
        u[acc] = un[better]
        F[acc] = Fn[better]
        e[acc] = en[better]
        lam[acc] = np.maximum(lam[acc] / 3.0, 1e-7)
        lam[idx[~better]] = np.minimum(lam[idx[~better]] * 4.0, 1e8)
        rejects[acc] = 0
        rejects[idx[~better]] += 1
        done = (better & (gain < rtol)) | (rejects[idx] >= 4)
        active[idx[done]] = False
    return FitResult(params=phys(u, np.arange(n)), curves=F, error=e, sims=sims, iterations=its,
                     seconds=time.perf_counter() - t0)


def surrogate_fit(sur: Surrogate, targets: np.ndarray, indenter_radius: np.ndarray, proto: Protocol,
                  max_iter: int = 8, starts: int = 16, inner_steps: int = 300, lr: float = 1e-2, rtol: float = 1e-3,
                  stats: SimStats | None = None, simulate=None) -> FitResult:
    """Surrogate-assisted fit. Proposals from the network (no simulation); then per iteration one
    verifying simulation of every active target and a defect-corrected refit of the network's
    inputs: with d = F_sim(p) - F_net(p) at the current point p, the inputs are refitted (Adam
    through the network, starting at p) so that F_net matches T - d. A target keeps its best
    simulated point and stops when an iteration improves its simulated error by less than rtol
    relative (or makes it worse)."""
    sim = simulate if simulate is not None else simulate_curves
    t0 = time.perf_counter()
    T = np.asarray(targets, np.float64).reshape(-1, proto.n_depths)
    n = T.shape[0]
    p = sur.propose(T, indenter_radius, starts=starts)
    best_p = p.copy()
    best_F = np.full_like(T, np.nan)
    best_e = np.full(n, np.inf)
    sims = np.zeros(n, np.int64)
    its = np.zeros(n, np.int64)
    active = np.ones(n, bool)
    scale = force_scale(proto)
    lo_u, hi_u = -np.ones(N_IN, np.float32), np.ones(N_IN, np.float32)
    for _ in range(max_iter):
        idx = np.flatnonzero(active)
        if idx.size == 0:
            break
        F = sim(p[idx], proto, stats)
        sims[idx] += 1
        its[idx] += 1
        e = curve_error(F, T[idx])
        e[~np.isfinite(e)] = np.inf
        improved = e < best_e[idx] * (1.0 - rtol)
        better = e < best_e[idx]
        upd = idx[better]
        best_p[upd], best_F[upd], best_e[upd] = p[upd], F[better], e[better]
        active[idx[~improved]] = False
        go = idx[improved]
        if go.size == 0:
            break
        d = F[improved] - sur.predict(p[go])                 # simulator - network at the current point
        y = ((T[go] - d) / scale).astype(np.float32)
        w = (1.0 / np.maximum((T[go] / scale) ** 2, 1e-300).sum(1)).astype(np.float32)
        u = to_unit(p[go], proto).astype(np.float32)
        rows = sur.net.max_batch
        for a in range(0, go.size, rows):
            u[a:a + rows], _ = sur.net.fit_inputs(u[a:a + rows], y[a:a + rows], FREE_MATERIAL, lo_u, hi_u,
                                                  steps=inner_steps, lr=lr, weight=w[a:a + rows])
        q = from_unit(u, proto)
        q[:, 5] = p[go, 5]  # the known radius stays exact
        p[go] = q
    return FitResult(params=best_p, curves=best_F, error=best_e, sims=sims, iterations=its,
                     seconds=time.perf_counter() - t0)


# The full experiment: a radius-16 cell (103,536 tetra), 48,000 steps per curve at 1e-4 per
# step. The small one (radius 8, 13,056 tetra, 2,400 steps) is for tests and quick checks.
FULL = Protocol()
SMALL = Protocol(radius=8.0, speed=1e-3, record_every=20, max_cells=4096)


def _stats(x: np.ndarray) -> dict:
    x = np.asarray(x, np.float64)
    x = x[np.isfinite(x)]
    if x.size == 0:
        return {"n": 0}
    return {"n": int(x.size), "mean": float(x.mean()), "median": float(np.median(x)),
            "p90": float(np.quantile(x, 0.9)), "max": float(x.max())}


def speed_sensitivity(P: np.ndarray, F: np.ndarray, proto: Protocol, alt_speed: float) -> dict:
    """How much the curves depend on the indentation speed: the inputs P (whose curves at
    proto.speed are F) simulated again at alt_speed, curve against curve at the same depths."""
    from dataclasses import replace

    alt = replace(proto, speed=alt_speed, record_every=max(10, int(round(proto.record_every * proto.speed / alt_speed))))
    Fa = simulate_curves(P, alt)
    ok = np.all(np.isfinite(F), axis=1) & np.all(np.isfinite(Fa), axis=1)
    d = curve_error(Fa[ok], F[ok])
    return {"speed": proto.speed, "alt_speed": alt_speed, "curves": int(ok.sum()), "relative_difference": _stats(d)}


def run_experiment(proto: Protocol = FULL, n_curves: int = 8192, n_hold: int = 1024, n_targets: int = 1024,
                   n_plain: int = 128, noise: float = 0.01, train_steps: int = 20000, batch: int = 512,
                   lr: float = 2e-3, starts: int = 16, seed: int = 0, log=print, data_out: str | None = None,
                   speed_check: int = 0, alt_speed: float = 5e-4) -> dict:
    """Curves from the batched simulator -> surrogate training -> held-out error -> inverse fits
    of noisy targets with and without the surrogate. Returns a JSON-ready summary. speed_check > 0
    also simulates that many of the dataset's inputs at alt_speed (speed_sensitivity)."""
    t_all = time.perf_counter()
    st_data = SimStats()
    P = sample_params(n_curves, proto, seed)
    F = simulate_curves(P, proto, st_data)
    ok = np.all(np.isfinite(F), axis=1)
    log(f"dataset: {n_curves} curves in {st_data.seconds:.1f} s, {int((~ok).sum())} non-finite")
    speed = None
    if speed_check > 0:
        speed = speed_sensitivity(P[:speed_check], F[:speed_check], proto, alt_speed)
        log(f"speed sensitivity: median curve difference {speed['relative_difference'].get('median', float('nan')):.3e} "
            f"between {proto.speed:g} and {alt_speed:g} per step")
    tr = np.arange(n_curves - n_hold)
    ho = np.arange(n_curves - n_hold, n_curves)
    tr, ho = tr[ok[tr]], ho[ok[ho]]
    sur = Surrogate(proto, max_batch=1024, seed=seed)
    t0 = time.perf_counter()
    hist = sur.train(P[tr], F[tr], steps=train_steps, batch=batch, lr=lr, seed=seed)
    t_train = time.perf_counter() - t0
    e_hold = curve_error(sur.predict(P[ho]), F[ho])
    log(f"training: {train_steps} steps in {t_train:.1f} s; held-out curve error median {np.median(e_hold):.3e}")

    # noisy targets from hidden inputs (drawn until n_targets valid simulations exist: inputs past
    # the scheme's stability limit give no curve)
    st_t = SimStats()
    Ph = sample_params(int(n_targets * 1.3) + 8, proto, seed + 1)
    Fh = simulate_curves(Ph, proto, st_t)
    valid = np.flatnonzero(np.all(np.isfinite(Fh), axis=1))[:n_targets]
    Ph, Fh = Ph[valid], Fh[valid]
    rng = np.random.default_rng(seed)
    T = Fh * (1.0 + noise * rng.standard_normal(Fh.shape))
    good = np.all(np.isfinite(T), axis=1)
    T, Ph, Fh = T[good], Ph[good], Fh[good]

    st_s = SimStats()
    rs = surrogate_fit(sur, T, Ph[:, 5], proto, starts=starts, stats=st_s)
    log(f"surrogate-assisted fit: {T.shape[0]} targets, {rs.sims.mean():.2f} simulations each, "
        f"median error {np.median(rs.error):.3e}")
    k = min(n_plain, T.shape[0])
    start = from_unit(np.zeros((k, N_IN)), proto)
    start[:, 5] = Ph[:k, 5]
    st_p = SimStats()
    rp = lm_fit(T[:k], start, proto, stats=st_p)
    log(f"plain fit: {k} targets, {rp.sims.mean():.2f} simulations each, median error {np.median(rp.error):.3e}")
    agree = curve_error(rs.curves[:k], rp.curves)
    sur.close()
    if data_out:
        np.savez_compressed(data_out, params=P, curves=F, target_params=Ph, targets=T, depths=proto.depths())
    noise_floor = curve_error(Fh, T)
    return {
        "protocol": {"radius": proto.radius, "speed": proto.speed, "steps": proto.steps, "n_depths": proto.n_depths,
                     "max_depth": proto.max_depth, "tets": int(proto.mesh().num_tetra)},
        "dataset": {"curves": n_curves, "non_finite": int((~ok).sum()), "sim_seconds": st_data.seconds,
                    "tetra_steps_per_s": st_data.tetra_steps / max(st_data.seconds, 1e-9)},
        "training": {"train_curves": int(tr.size), "steps": train_steps, "batch": batch, "seconds": t_train,
                     "final_loss": float(np.mean(hist[-100:])) if hist is not None and hist.size else None},
        "held_out_curve_error": _stats(e_hold),
        "inverse_fit": {
            "targets": int(T.shape[0]), "noise": noise, "noise_floor_error": _stats(noise_floor),
            "surrogate": {"sims_per_target": float(rs.sims.mean()), "seconds_per_target": rs.seconds / T.shape[0],
                          "error": _stats(rs.error)},
            "plain": {"targets": k, "sims_per_target": float(rp.sims.mean()), "seconds_per_target": rp.seconds / k,
                      "error": _stats(rp.error)},
            "sims_ratio_plain_over_surrogate": float(rp.sims.mean() / max(rs.sims[:k].mean(), 1e-9)),
            "wall_ratio_plain_over_surrogate": float((rp.seconds / k) / max(rs.seconds / T.shape[0], 1e-9)),
            "fit_curves_agree_within_1e-3": float(np.mean(agree <= 1e-3)),
            "surrogate_error_le_plain_plus_1e-3": float(np.mean(rs.error[:k] <= rp.error + 1e-3)),
            "agreement": _stats(agree),
        },
        "speed_sensitivity": speed,
        "wall_seconds": time.perf_counter() - t_all,
    }


def main(argv=None) -> int:
    import argparse
    import json

    ap = argparse.ArgumentParser(description="surrogate training and surrogate-assisted inverse fitting")
    ap.add_argument("--protocol", choices=["full", "small"], default="full")
    ap.add_argument("--curves", type=int, default=8192)
    ap.add_argument("--hold", type=int, default=1024)
    ap.add_argument("--targets", type=int, default=1024)
    ap.add_argument("--plain", type=int, default=128, help="targets also fitted by the plain method")
    ap.add_argument("--train-steps", type=int, default=20000)
    ap.add_argument("--batch", type=int, default=512)
    ap.add_argument("--seed", type=int, default=0)
    ap.add_argument("--out", default=None, help="JSON summary path")
    ap.add_argument("--data", default=None, help="npz path for the generated curves")
    ap.add_argument("--speed", type=float, default=None, help="indentation per step (default: the protocol's)")
    ap.add_argument("--speed-check", type=int, default=0,
                    help="dataset inputs also simulated at --alt-speed to measure the speed dependence")
    ap.add_argument("--alt-speed", type=float, default=5e-4)
    a = ap.parse_args(argv)
    proto = FULL if a.protocol == "full" else SMALL
    if a.speed is not None:
        from dataclasses import replace

        proto = replace(proto, speed=a.speed)
    res = run_experiment(proto, a.curves, a.hold, a.targets, a.plain, train_steps=a.train_steps, batch=a.batch,
                         seed=a.seed, data_out=a.data, speed_check=a.speed_check, alt_speed=a.alt_speed)
    text = json.dumps(res, indent=1)
    if a.out:
        with open(a.out, "w") as f:
            f.write(text + "\n")
    print(text)
    return 0


if __name__ == "__main__":
    raise SystemExit(main())
