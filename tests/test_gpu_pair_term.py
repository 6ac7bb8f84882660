"""The pair term (ScatterField.pp_acc, scripts/scatter_field.py:291-300, 324-364, 500-521) on the
GPU against the reference's own outputs (tests/golden/pair_acc.npz: dense, cell-list and adaptive
multilevel modes) and
the oracle's float64 brute-force top-knn, plus the edge cases of its cell list: masked bodies,
bodies outside the box (clamped cells), fewer than knn neighbours, a pair radius small enough
that the cells are coarsened, and order independence."""
import numpy as np
import pytest
import torch

from augur_gb300 import PMPlan
from oracle import pm_oracle as O

pytestmark = pytest.mark.gpu
DEV = torch.device("cuda:0")
CASES = ("dense", "cell", "cell_cu", "adapt")
TOL = 1e-4  # fp32 distances, features and MLP against float64 / the reference's fp32


def _case(golden, case):
    kg = golden["pair_acc"]
    return {k[len(case) + 1:]: kg[k] for k in kg.files if k.startswith(case + "_")}


def rel(a, b):
    return float(np.sqrt(((a - b) ** 2).sum() / max((b ** 2).sum(), 1e-300)))


def _run(plan, pos, mass, mask, g, params="golden", **kw):
    f = int(g["flags"])
    prm = torch.from_numpy(g["params"]).to(DEV) if isinstance(params, str) else params
    args = dict(ppe=float(g["ppe"]), knn=int(g["knn"]), params=prm, ncol=int(g["ncol"]),
                extra=g["extra"].tolist(), cell_units=bool(f & 1), prior=bool(f & 2), eps=float(g["eps"]))
    args.update(kw)
    t = lambda a: torch.as_tensor(np.ascontiguousarray(a), dtype=torch.float32, device=DEV)
    out = plan.pair_acc(t(pos), t(mass), t(mask), **args)
    plan.check()
    return out.cpu().numpy().astype(np.float64)


def _oracle(pos, mass, mask, g, params="golden", queries=None, **kw):
    f = int(g["flags"])
    a = dict(params=g["params"] if isinstance(params, str) else params, ncol=int(g["ncol"]),
             extra=g["extra"].tolist(), flags=f, ppe=float(g["ppe"]), eps=float(g["eps"]), h=float(g["h"]),
             knn=int(g["knn"]))
    a.update(kw)
    return O.pair_acc_2d(pos, mass, mask, queries=queries, **a)


def _plan(g, n):
    grid = int(round(float(g["extent"]) / float(g["h"])))
    return PMPlan(2, grid, max(1, n), "isolated", float(g["extent"]), eps=float(g["eps"]), device=DEV)


@pytest.mark.parametrize("case", CASES)
def test_pair_acc_matches_reference(golden, case):
    g = _case(golden, case)
    pos, mass, mask = g["pos"], g["mass"], g["mask"]
    plan = _plan(g, len(pos))
    acc = _run(plan, pos, mass, mask, g)
    assert rel(acc, g["acc"].astype(np.float64)) < TOL
    assert rel(acc, _oracle(pos, mass, mask, g)) < TOL
    assert np.all(acc[mask <= 0] == 0.0)


def test_pair_acc_prior_only_and_mlp_only_add_up(golden):
    g = _case(golden, "cell")
    pos, mass, mask = g["pos"], g["mass"], g["mask"]
    plan = _plan(g, len(pos))
    both = _run(plan, pos, mass, mask, g)
    prior = _run(plan, pos, mass, mask, g, params=None)
    mlp = _run(plan, pos, mass, mask, g, prior=False)
    assert rel(prior, _oracle(pos, mass, mask, g, params=None)) < TOL
    assert rel(prior + mlp, both) < 1e-5


def test_pair_acc_edges(golden):
    """Bodies outside the box, masked bodies, sparse bodies with fewer than knn neighbours
    inside the pair radius, knn = 1 and knn = 32."""
    g = _case(golden, "cell")
    E = float(g["extent"])
    rng = np.random.default_rng(71)
    n = 4000
    pos = np.concatenate([rng.normal(0, E / 8, (n - 400, 2)), rng.uniform(-0.7 * E, 0.7 * E, (400, 2))])
    pos = pos.astype(np.float32)
    mass = rng.uniform(0.5, 1.5, n).astype(np.float32)
    mask = (rng.uniform(size=n) > 0.1).astype(np.float32)
    plan = _plan(g, n)
    q = rng.choice(n, 300, replace=False)
    for knn in (1, 16, 32):
        acc = _run(plan, pos, mass, mask, g, knn=knn)
        ora = _oracle(pos, mass, mask, g, queries=q, knn=knn)
        assert rel(acc[q], ora[q]) < TOL, knn
        assert np.all(acc[mask <= 0] == 0.0)
    outside = np.abs(pos).max(1) > E / 2
    assert outside.sum() > 50 and np.abs(acc[outside & (mask > 0)]).sum() > 0


def test_pair_acc_coarsened_cells(golden):
    """ceil(extent / ppe) above the cell cap: the plan uses coarser cells, results unchanged."""
    g = _case(golden, "cell")
    E = float(g["extent"])
    ppe = E / 3000.0
    rng = np.random.default_rng(5)
    n = 20000
    pos = rng.uniform(-E / 64, E / 64, (n, 2)).astype(np.float32)  # dense enough for pairs within ppe
    mass = np.ones(n, np.float32)
    mask = np.ones(n, np.float32)
    plan = _plan(g, n)
    acc = _run(plan, pos, mass, mask, g, ppe=ppe)
    q = rng.choice(n, 200, replace=False)
    ora = _oracle(pos, mass, mask, g, queries=q, ppe=ppe)
    assert np.abs(ora[q]).sum() > 0
    assert rel(acc[q], ora[q]) < TOL


def test_pair_acc_is_order_independent(golden):
    """Neighbours are summed in ascending (distance, index) order: repeated calls are identical,
    and a permutation of the bodies permutes the output bit for bit wherever no two neighbours of
    a body are at the same fp32 distance (the index then decides their order)."""
    g = _case(golden, "cell_cu")
    E = float(g["extent"])
    rng = np.random.default_rng(9)
    n = 50000
    pos = rng.uniform(-E / 2, E / 2, (n, 2)).astype(np.float32)
    mass = rng.uniform(0.5, 1.5, n).astype(np.float32)
    mask = np.ones(n, np.float32)
    plan = _plan(g, n)
    a = _run(plan, pos, mass, mask, g)
    b = _run(plan, pos, mass, mask, g)
    assert np.array_equal(a, b)
    perm = rng.permutation(n)
    c = _run(plan, pos[perm], mass[perm], mask[perm], g)
    same = (c == a[perm]).all(1)
    assert same.mean() > 0.999, same.mean()
    assert rel(c, a[perm]) < 1e-6


def test_pair_acc_rejects_bad_arguments(golden):
    g = _case(golden, "cell")
    plan = _plan(g, 10)
    pos = torch.zeros((10, 2), device=DEV)
    with pytest.raises(RuntimeError):
        plan.pair_acc(pos, ppe=2.0, knn=33)
    with pytest.raises(RuntimeError):
        plan.pair_acc(pos, ppe=0.0)
    p3 = PMPlan(3, 32, 10, "periodic", 1.0, device=DEV)
    with pytest.raises(RuntimeError):
        p3.pair_acc(torch.zeros((10, 3), device=DEV))
