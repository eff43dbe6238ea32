"""Small parity cases shared by the golden-vector generator, the oracle tests and the GPU tests.

Each case is a workload plus overrides. The meshes come from mesh.kuhn_sphere with a fixed
seed (numpy's PCG64 stream is the same on every platform), so only outputs are stored.
"""

from __future__ import annotations

from dataclasses import dataclass

import oracle as O
from nofluidx3d_gb300.workloads import Workload


@dataclass
class Case:
    name: str
    workload: Workload
    steps: int
    model: int | None = None        # override of the elastic model (O.MODEL_SVK / O.MODEL_SVKK)
    fix_top_bottom: bool = False

    def problem(self) -> O.Problem:
        from tests.helpers import oracle_problem

        p = oracle_problem(self.workload)
        if self.model is not None:
            p.model = self.model
        p.fix_top_bottom = self.fix_top_bottom
        return p


def _w(**kw) -> Workload:
    base = dict(name="golden", radius=3.0, speed=1e-3, record_every=50, steps=300)
    base.update(kw)
    return Workload(**base)


CASES = {
    c.name: c
    for c in [
        Case("nh_plane_R3", _w(material="nh"), 300),
        Case("mr_plane_R3", _w(material="mr"), 300),
        Case("vp_sphere_R3", _w(material="mr_vp", indenter="sphere", sphere_radius=2.0), 300),
        Case("svk_plane_R3", _w(material="nh"), 200, model=O.MODEL_SVK),
        Case("svkk_plane_R3", _w(material="nh"), 200, model=O.MODEL_SVKK),
        Case("nh_fixtb_R3", _w(material="nh"), 200, fix_top_bottom=True),
        Case("mr_vv2_sphere_R3", _w(material="mr", indenter="sphere", sphere_radius=2.0, integrator="vv2",
                                    xi=0.05), 300),
        Case("mr_sphereint_R3", _w(material="mr", indenter="sphere_integral", sphere_radius=2.0, d0=0.3), 300),
        Case("vp_sphereint_vv2_R3", _w(material="mr_vp", indenter="sphere_integral", sphere_radius=2.0, d0=0.3,
                                       integrator="vv2", xi=0.05), 300),
    ]
}
