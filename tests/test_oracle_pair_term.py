"""The oracle's restatement of the pair term (ScatterField.pp_acc, scripts/scatter_field.py:291-300,
324-471, 500-521) against the reference's own outputs (tests/golden/pair_acc.npz: dense mode, the
cell-list mode with plain and cell-unit features, and the adaptive multilevel mode). No GPU."""
import numpy as np
import pytest

from oracle import pm_oracle as O

CASES = ("dense", "cell", "cell_cu", "adapt")


def _case(golden, case):
    kg = golden["pair_acc"]
    return {k[len(case) + 1:]: kg[k] for k in kg.files if k.startswith(case + "_")}


@pytest.mark.parametrize("case", CASES)
def test_oracle_pair_acc_matches_reference(golden, case):
    g = _case(golden, case)
    acc = O.pair_acc_2d(g["pos"], g["mass"], g["mask"], g["params"], int(g["ncol"]), g["extra"].tolist(),
                        int(g["flags"]), float(g["ppe"]), float(g["eps"]), float(g["h"]), int(g["knn"]))
    ref = g["acc"].astype(np.float64)
    err = np.sqrt(((acc - ref) ** 2).sum() / (ref ** 2).sum())
    assert err < 1e-5, err
