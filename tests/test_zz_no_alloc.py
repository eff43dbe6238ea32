"""nfx_indenter_force_noalloc — the readout for callers that cannot allocate device memory.

Some callers keep node positions in device buffers they own and may not allocate (their own
memory pool reserves the whole device budget, or their time loop must not allocate). The
no-alloc readout keeps its reduction scratch in a static device array instead of handle
memory. Here it is called through the C ABI on positions held in caller-owned device memory
and compared with the handle's own readout, nfx_indenter_force, on two calls in a row (the
cell advanced between them), for a flat and a spherical indenter and for the substrate under the
cell (whose force has the opposite sign). This file is collected last
so that a stop at the first failure has already run every other test; it does not depend on
them and passes in a fresh process too.
"""

import pytest

pytestmark = pytest.mark.gpu

RTOL = 1e-12  # both are fixed-order FP64 reductions of the same terms, summed in different orders


@pytest.mark.parametrize("name,contact", [("nh_plane_R3", 1), ("vp_sphere_R3", 1), ("vp_sphere_R3", 0)],
                         ids=["plane", "sphere", "substrate"])
def test_noalloc_readout_matches_handle_readout_twice(name, contact):
    import torch

    from nofluidx3d_gb300 import _lib
    from nofluidx3d_gb300.core import CellSim
    from tests.golden.cases import CASES

    L = _lib.load()
    w = CASES[name].workload
    sim = CellSim(0)
    w.configure(sim)
    c = w.contacts()[contact]
    out = torch.zeros(2, dtype=torch.float64, device="cuda:0")
    for call in range(2):
        sim.step(100)
        expected = sim.indenter_force(contact)
        assert expected != 0.0
        pts = torch.from_numpy(sim.points_soa()).to("cuda:0")
        position = c["p0"] - c["v"] * min(sim.time, c["tmove"])
        torch.cuda.synchronize()
        _lib.check(L.nfx_indenter_force_noalloc(0, sim.np, pts.data_ptr(), c["kind"], c["k"], c["radius"], position,
                                                out[call].data_ptr(), None))
        torch.cuda.synchronize()
        assert out[call].item() == pytest.approx(expected, rel=RTOL, abs=0.0)
    sim.close()


def test_noalloc_rejects_sizes_beyond_its_scratch():
    import torch

    from nofluidx3d_gb300 import _lib

    L = _lib.load()
    pts = torch.zeros(3, dtype=torch.float64, device="cuda:0")
    out = torch.zeros(1, dtype=torch.float64, device="cuda:0")
    too_many = 4194304 + 1
    rc = L.nfx_indenter_force_noalloc(0, too_many, pts.data_ptr(), 1, 0.1, 0.0, 0.0, out.data_ptr(), None)
    assert rc == 1
    assert "4194304" in _lib.last_error()
