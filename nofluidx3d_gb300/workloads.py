"""Indentation workloads in lattice units, and their set-up on a CellSim.

Each workload is one cell: a Kuhn-split sphere (mesh.kuhn_sphere) resting on a rigid substrate
at y = -(R + d0), indented from above by a flat plane or a sphere descending at `speed` per
step, integrated by damped velocity Verlet with dt = 1 and unit nodal mass, penalty constant
k for every contact (Simulation.py:106-230 sets the same interactions from a JSON config).

Material mapping to the reference's parameters:
  * Neo-Hookean with shear modulus mu and bulk modulus K is Tetra(E, nu, mooneyRivlinRatio=1)
    with E = 9 K mu / (3 K + mu), nu = (3 K - 2 mu) / (2 (3 K + mu)); tetra.cl:118-121 then
    recovers mu = E / (2 (1 + nu)) and kappa = E / (3 (1 - 2 nu)) = K.
  * Mooney-Rivlin C10, C01 is mu1 = 2 C10, mu2 = 2 C01.
  * "yield stress Y, plastic viscosity eta" maps onto the reference's power-law flow rule
    (InteractionFiniteStrainViscoplastic.cl:149-153) with flowExponent m = 1, no hardening
    (hardeningExponent 0, threshold 1) and plasticFlowRate = Y / eta, so the plastic
    stretch rate is sigma_vm / eta.
"""

from __future__ import annotations

from dataclasses import dataclass, field, replace

from .mesh import CellMesh, kuhn_sphere

__all__ = ["Workload", "plain_small", "plain_large", "plain_large_1m", "nh_to_reference", "WORKLOADS"]


def nh_to_reference(mu: float, K: float) -> tuple[float, float]:
    """(E, nu) of Tetra for a Neo-Hookean shear modulus mu and bulk modulus K."""
    E = 9.0 * K * mu / (3.0 * K + mu)
    nu = (3.0 * K - 2.0 * mu) / (2.0 * (3.0 * K + mu))
    return E, nu


@dataclass
class Workload:
    name: str
    radius: float
    material: str = "nh"        # "nh", "mr" or "mr_vp"
    mu: float = 1e-3            # NH shear modulus
    K: float = 1e-2             # bulk modulus
    C10: float = 5e-4
    C01: float = 1e-4
    yield_stress: float = 2e-4
    viscosity: float = 5e-2
    indenter: str = "plane"     # "plane", "sphere" or "sphere_integral" (InteractionSphereIntegral.cl)
    sphere_radius: float = 16.0
    speed: float = 1e-4
    d0: float | None = 0.0      # InitialDistance; None: top node's height - radius (see initial_distance)
    k: float = 0.1              # def_FORCE_CONST
    si_k: float = 12.0          # PotentialForceConst of the integrated sphere contact (decay rate)
    xi: float = 1e-2            # velocity damping
    integrator: str = "vv"      # "vv" (VelocityVerlet.cl, unit mass) or "vv2" (velocityVerlet2.cl)
    density: float = 1.0        # lumped masses of "vv2"
    steps: int = 20000
    record_every: int = 100
    jitter: float = 0.02
    seed: int = 0
    extra: dict = field(default_factory=dict)

    def mesh(self) -> CellMesh:
        return kuhn_sphere(self.radius, self.jitter, self.seed)

    # reference-style parameters -------------------------------------------------------
    def tetra_params(self) -> tuple[int, float, float, float]:
        """(model, E, nu, mooneyRivlinRatio) of the elastic Tetra plugin."""
        if self.material == "nh":
            E, nu = nh_to_reference(self.mu, self.K)
            return 0, E, nu, 1.0
        mu1, mu2 = 2.0 * self.C10, 2.0 * self.C01
        E, nu = nh_to_reference(mu1 + mu2, self.K)
        return 0, E, nu, mu1 / (mu1 + mu2)

    def vp_params(self) -> tuple[float, ...]:
        """{mu1, mu2, kappa, flowExponent, yieldStress, plasticFlowRate, hardeningThreshhold,
        hardeningExponent} of the viscoplastic law."""
        return (2.0 * self.C10, 2.0 * self.C01, self.K, 1.0, self.yield_stress,
                self.yield_stress / self.viscosity, 1.0, 0.0)

    def initial_distance(self, mesh: CellMesh | None = None) -> float:
        """InitialDistance of the walls (Simulation.py:107, :118, :162). With d0 = None it is the
        top node's height above the radius, so that the substrate (at -(R + d0)) and the indenter
        (at R + d0, plus the sphere radius) start tangent to the mesh's lowest and highest nodes
        (nodes 4 and 3, which the Kuhn sphere places symmetrically). A lattice sphere of
        non-integer radius has its top node up to one spacing above R: walls placed at +-R would
        start inside the mesh and kick soft cells apart on the first step."""
        if self.d0 is not None:
            return float(self.d0)
        if mesh is None:
            raise ValueError("d0 = None needs the mesh to place the walls")
        return float(mesh.points[3, 1]) - self.radius

    def contacts(self, mesh: CellMesh | None = None) -> list[dict]:
        """Substrate first, then the indenter (the recorded contact, index 1)."""
        R = self.radius
        d0 = self.initial_distance(mesh)
        out = [dict(kind=0, k=self.k, radius=0.0, p0=-(R + d0), v=0.0, tmove=float("inf"))]
        if self.indenter == "plane":
            out.append(dict(kind=1, k=self.k, radius=0.0, p0=R + d0, v=self.speed, tmove=float("inf")))
        elif self.indenter == "sphere":
            Rs = self.sphere_radius
            out.append(dict(kind=2, k=self.k, radius=Rs, p0=R + Rs + d0, v=self.speed, tmove=float("inf")))
        elif self.indenter == "sphere_integral":
            Rs = self.sphere_radius
            out.append(dict(kind=3, k=self.si_k, radius=Rs, p0=R + Rs + d0, v=self.speed, tmove=float("inf")))
        else:
            raise ValueError(f"unknown indenter {self.indenter!r}")
        return out

    def set_integrator_on(self, target, cell=None) -> None:
        """The integrator on a CellSim (cell None) or on one cell of a Batch."""
        args = () if cell is None else (cell,)
        if self.integrator == "vv2":
            target.set_integrator_lumped(*args, self.xi, self.density)
        elif self.integrator == "vv":
            target.set_integrator(*args, self.xi, False)
        else:
            raise ValueError(f"unknown integrator {self.integrator!r}")

    @property
    def record_contact(self) -> int:
        return 1

    def configure(self, sim, mesh: CellMesh | None = None, max_rows: int | None = None) -> CellMesh:
        """Set mesh, material, contacts, integrator and recording on a CellSim."""
        m = mesh if mesh is not None else self.mesh()
        sim.set_mesh(m.points, m.tets)
        if self.material == "mr_vp":
            sim.set_viscoplastic(self.vp_params())
        else:
            model, E, nu, mr = self.tetra_params()
            sim.set_tetra(model, E, nu, mr)
        for c in self.contacts(m):
            sim.add_contact(c["kind"], c["k"], c["radius"], c["p0"], c["v"], c["tmove"])
        self.set_integrator_on(sim)
        rows = max_rows if max_rows is not None else self.steps // self.record_every + 1
        sim.set_record(self.record_contact, self.record_every, rows)
        return m

    def add_to_batch(self, batch, mesh: CellMesh | None = None, like: int | None = None) -> int:
        """Add this cell (mesh, material, contacts, integrator) to a core.Batch; returns its index.
        like: index of a cell already in the batch whose mesh (which must be `mesh`) is shared."""
        m = mesh if mesh is not None else self.mesh()
        cell = batch.add_cell(m.points, m.tets) if like is None else batch.add_cell_like(like)
        if self.material == "mr_vp":
            batch.set_viscoplastic(cell, self.vp_params())
        else:
            model, E, nu, mr = self.tetra_params()
            batch.set_tetra(cell, model, E, nu, mr)
        for c in self.contacts(m):
            batch.add_contact(cell, c["kind"], c["k"], c["radius"], c["p0"], c["v"], c["tmove"])
        self.set_integrator_on(batch, cell)
        return cell

    def with_(self, **kw) -> "Workload":
        return replace(self, **kw)


def plain_small() -> Workload:
    """R = 8 Neo-Hookean cell, flat indenter, 20k steps (13,056 tetra, 2,849 nodes)."""
    return Workload("plain-small R8 NH plane", radius=8.0, material="nh", mu=1e-3, K=1e-2, indenter="plane",
                    steps=20000)


def plain_large() -> Workload:
    """R = 64 Mooney-Rivlin + viscoplastic cell, sphere indenter of radius 16, 50k steps
    (6,594,816 tetra, 1,138,197 nodes)."""
    return Workload("plain-large R64 MR+VP sphere", radius=64.0, material="mr_vp", C10=5e-4, C01=1e-4, K=1e-2,
                    yield_stress=2e-4, viscosity=5e-2, indenter="sphere", sphere_radius=16.0, steps=50000)


def plain_large_1m() -> Workload:
    """The same construction at R = 34, the radius that gives ~1M tetra (989,808 tetra,
    176,093 nodes)."""
    return plain_large().with_(name="plain-large R34 MR+VP sphere", radius=34.0)


def plain_large_r48() -> Workload:
    """The same construction at R = 48 (2,780,400 tetra): large enough that one step's
    viscoplastic state (~350 MB read + written) exceeds L2, small enough for full ncu captures."""
    return plain_large().with_(name="plain-large R48 MR+VP sphere", radius=48.0)


WORKLOADS = {"plain-small": plain_small, "plain-large": plain_large, "plain-large-1m": plain_large_1m,
             "plain-large-r48": plain_large_r48}


def batched_cells(n: int = 256, seed: int = 0, r_range=(6.0, 40.0), steps: int = 20000) -> list[Workload]:
    """The batched population: n cells with radius log-uniform in r_range, per-cell jitter seed
    (seed + cell index), and per-cell material drawn log-uniform — shear modulus 2e-4..5e-3,
    bulk/shear ratio 5..50, yield stress 5e-5..1e-3, plastic viscosity 1e-2..1e-1 — with the
    viscoplastic law (elastic part Neo-Hookean: mu1 = shear modulus, mu2 = 0). Each cell rests
    on a substrate and is indented by a sphere of a quarter of its radius at 1e-4 per step; the
    walls start tangent to the cell's top and bottom nodes (d0 = None)."""
    import numpy as np

    rng = np.random.default_rng(seed)

    def logu(lo, hi, size):
        return np.exp(rng.uniform(np.log(lo), np.log(hi), size))

    R = logu(*r_range, n)
    mu = logu(2e-4, 5e-3, n)
    ratio = logu(5.0, 50.0, n)
    Y = logu(5e-5, 1e-3, n)
    eta = logu(1e-2, 1e-1, n)
    out = []
    for i in range(n):
        out.append(Workload(f"batched cell {i}", radius=float(R[i]), material="mr_vp", C10=float(mu[i]) / 2.0,
                            C01=0.0, K=float(mu[i] * ratio[i]), yield_stress=float(Y[i]), viscosity=float(eta[i]),
                            indenter="sphere", sphere_radius=float(R[i]) / 4.0, steps=steps, seed=seed + i,
                            d0=None))
    return out
