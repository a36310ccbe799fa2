"""Pressure boundaries in the oracle's calcp_simple (facefluxmassPressBnd,
faceflux_mass.f90:765-830, before the pressure-correction solve;
facefluxmassCorrPressBnd, :699-762, after it; p' = 0 at the boundary and as
the reference value, calcp_simple.f90:162-183,344-369): on a channel with a
velocity inlet and a p = 0 outlet, the mass leaving through the pressure
patch equals the mass entering, p' is zero on the patch, and the prescribed
boundary pressure stays in place."""
import numpy as np

from channel_cases import channel, patch_flux


def test_channel_with_pressure_outlet_conserves_mass(oracle):
    m, a, oc, prm = channel(oracle)
    nC, nI = m.numCells, m.numInnerFaces
    for _ in range(120):
        st, res, _ = oc.simple_iteration()
        assert st >= 0
    fm = oc.get("flmass")
    fin, fout = patch_flux(a, fm, 0), patch_flux(a, fm, 1)
    assert fin == -1.0 or abs(fin + 1.0) < 1e-12   # inlet fluxes as prescribed (area 1, u = 1)
    assert abs(fin + fout) < 1e-8
    b1 = a["startFace"][1] - nI
    sl = slice(nC + b1, nC + b1 + a["nfaces"][1])
    assert np.all(oc.get("pp")[sl] == 0.0)
    assert np.all(oc.get("p")[sl] == 0.0)
    # the momentum residuals have fallen from O(1)
    assert max(res[:3]) < 1e-6
