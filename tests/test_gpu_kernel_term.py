"""The learned kernel term (ScatterField.kernel_acc, scripts/scatter_field.py:263-289) on the GPU
against the reference's own outputs (tests/golden/kernel_acc.npz) and the oracle."""
import numpy as np
import pytest
import torch

from augur_gb300 import PMPlan
from oracle import pm_oracle as O

pytestmark = pytest.mark.gpu
DEV = torch.device("cuda:0")
CASES = ("plain", "split_ext", "cu_prior")


def _case(golden, case):
    kg = golden["kernel_acc"]
    return {k[len(case) + 1:]: kg[k] for k in kg.files if k.startswith(case + "_")}


def _plan(g):
    plan = PMPlan(2, int(g["grid"]), 1, "isolated", float(g["extent"]), eps=float(g["eps"]), device=DEV)
    f = int(g["flags"])
    plan.set_kernel_mlp(torch.from_numpy(g["params"]).to(DEV), int(g["ncol"]), g["extra"].tolist(),
                        cell_units=bool(f & 1), prior=bool(f & 2), split=bool(f & 4),
                        split_radius=float(g["split_radius"]), eps=float(g["eps"]), pad_ext=bool(f & 8))
    return plan


def rel(a, b):
    return float(np.sqrt(((a - b) ** 2).sum() / (b ** 2).sum()))


@pytest.mark.parametrize("case", CASES)
def test_kernel_acc_matches_reference(golden, case):
    g = _case(golden, case)
    plan = _plan(g)
    F4 = plan.poisson(torch.from_numpy(g["rho"]).to(DEV)).cpu().numpy()
    plan.check()
    assert rel(F4[..., :2].astype(np.float64), g["acc"].astype(np.float64)) < 1e-4
    # the oracle (float64) agrees as closely
    ora = O.kernel_acc_2d(g["rho"], g["params"], int(g["ncol"]), g["extra"].tolist(), int(g["flags"]),
                          float(g["split_radius"]), float(g["eps"]), float(g["extent"]))
    assert rel(F4[..., :2].astype(np.float64), ora) < 1e-4


def test_reset_kernel_restores_plain_pm(golden):
    g = _case(golden, "split_ext")
    plan = _plan(g)
    rho = torch.from_numpy(g["rho"]).to(DEV)
    learned = plan.poisson(rho).clone()
    plan.reset_kernel()
    plain = plan.poisson(rho)
    ref = PMPlan(2, int(g["grid"]), 1, "isolated", float(g["extent"]), eps=float(g["eps"]), device=DEV).poisson(rho)
    assert torch.equal(plain, ref)
    assert not torch.allclose(learned, plain)


def test_kernel_params_are_validated():
    plan = PMPlan(2, 32, 1, "isolated", 64.0, eps=0.5, device=DEV)
    with pytest.raises(ValueError):
        plan.set_kernel_mlp(torch.zeros(100), 2)
    with pytest.raises(RuntimeError):  # split needs a radius
        plan.set_kernel_mlp(torch.zeros(64 * 2 + 64 * 64 + 3 * 64 + 1), 2, split=True)
    per = PMPlan(3, 32, 1, "periodic", 1.0, device=DEV)
    with pytest.raises(RuntimeError):  # periodic plans have no lattice kernel
        per.set_kernel_mlp(torch.zeros(64 * 2 + 64 * 64 + 3 * 64 + 1), 2)
