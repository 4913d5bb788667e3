"""GPU parity of the Smargiassi-Madden and Perrot kinetic functionals (kedf/sm.py,
fp.py) against the reference's outputs (tests/golden/make_golden_wtfam.py):
energy within 1e-10 relative, potential within 1e-9 and stress within 1e-9 of
their largest values in FP64; FP32 energy within 2e-6 relative."""
import os

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

import dftpy_gb300 as D

HERE = os.path.dirname(os.path.abspath(__file__))
WF = dict(np.load(os.path.join(HERE, "golden", "reference_wtfam.npz")))
CASES = [("SM", "SM", {}), ("FP", "FP", {}), ("SMNL", "SM-NL", {}), ("SMA", "SM", {"alpha": 0.6, "beta": 0.6})]


def _np(f):
    return f.as_subclass(torch.Tensor).double().cpu().numpy()


@pytest.mark.parametrize("tag,name,kw", CASES, ids=[c[0] for c in CASES])
def test_wt_family_against_reference(golden, tag, name, kw):
    grid = D.DirectGrid(golden["A_lattice"], golden["A_nr"])
    rho = D.DirectField(grid, data=golden["A_rho"])
    f = D.Functional(type="KEDF", name=name, **kw)
    o = f(rho)
    e, v, s = WF["A_E_" + tag], WF["A_V_" + tag], WF["A_S_" + tag]
    assert abs(o.energy - e) <= 1e-10 * abs(e), (o.energy, e)
    assert float(np.abs(_np(o.potential) - v).max()) <= 1e-9 * float(np.abs(v).max())
    st = f.stress(rho)
    assert float(np.abs(st - s).max()) <= 1e-9 * float(np.abs(s).max())
    o32 = f(D.DirectField(grid, data=golden["A_rho"], dtype=torch.float32))
    assert abs(o32.energy - e) <= 2e-6 * abs(e)
