"""The oracle's restatement of the learned kernel term (ScatterField.kernel_acc,
scripts/scatter_field.py:263-289) against the reference's own outputs (tests/golden/kernel_acc.npz,
made by tests/golden/make_golden.py with seeded kmlp weights). No GPU."""
import numpy as np
import pytest

from oracle import pm_oracle as O

CASES = ("plain", "split_ext", "cu_prior")


@pytest.fixture(scope="module")
def kgold(golden):
    return golden["kernel_acc"]


@pytest.mark.parametrize("case", CASES)
def test_oracle_kernel_acc_matches_reference(kgold, case):
    g = {k[len(case) + 1:]: kgold[k] for k in kgold.files if k.startswith(case + "_")}
    acc = O.kernel_acc_2d(g["rho"], g["params"], int(g["ncol"]), g["extra"].tolist(), int(g["flags"]),
                          float(g["split_radius"]), float(g["eps"]), float(g["extent"]))
    ref = g["acc"].astype(np.float64)
    err = np.sqrt(((acc - ref) ** 2).sum() / (ref ** 2).sum())
    # the reference evaluates in float32; its rounding of the potential before the central
    # difference (O(1/r) values differenced across two cells) is the difference seen here
    assert err < 1e-4, err
