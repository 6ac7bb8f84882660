"""The allocation-free FP64 direct sum (augur_direct_sum_fp64_noalloc), called through the C
ABI, against the allocating entry point (augur_direct_sum_fp64) on two calls in a row.

It serves callers that cannot allocate device memory: work issued during CUDA stream capture,
and processes whose device memory another allocator already holds. Its scratch is a static
device array shared by all calls, so the second call also checks that nothing stale from the
first one leaks into it. This file is collected last on purpose."""
import ctypes as C

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu
DEV = torch.device("cuda:0")
TOL = 1e-12  # relative: same pair sums, different order of the per-chunk partials


def _lib():
    from augur_gb300 import _lib as L

    return L.load()


def _call(name, targets, tidx, sources, mass, dim, eps, out, box=None):
    lib = _lib()
    stream = torch.cuda.current_stream(DEV).cuda_stream
    args = [C.c_void_p(targets.data_ptr()), C.c_void_p(tidx.data_ptr()), C.c_int64(targets.shape[0]),
            C.c_void_p(sources.data_ptr()), C.c_void_p(mass.data_ptr()), C.c_int64(sources.shape[0]),
            C.c_int(dim), C.c_double(eps)]
    if box is not None:
        args.append(C.c_double(box))
    args += [C.c_void_p(out.data_ptr()), C.c_void_p(stream)]
    return getattr(lib, name)(*args)


@pytest.mark.parametrize("dim,n,t", [(3, 200000, 3000), (2, 50000, 700)])
def test_noalloc_matches_allocating_direct_sum_twice(dim, n, t):
    for call in range(2):
        g = torch.Generator().manual_seed(100 * dim + call)
        src = (torch.randn(n, dim, generator=g, dtype=torch.float64) * 0.1).to(DEV)
        mass = (torch.rand(n, generator=g, dtype=torch.float64) + 0.5).to(DEV)
        idx = torch.randperm(n, generator=g)[:t].to(DEV)
        tg = src[idx].contiguous()
        ref = torch.empty(t, dim, dtype=torch.float64, device=DEV)
        out = torch.full((t, dim), float("nan"), dtype=torch.float64, device=DEV)
        assert _call("augur_direct_sum_fp64", tg, idx, src, mass, dim, 1e-3, ref, box=0.0) == 0
        assert _call("augur_direct_sum_fp64_noalloc", tg, idx, src, mass, dim, 1e-3, out) == 0
        torch.cuda.synchronize()
        a, b = out.cpu().numpy(), ref.cpu().numpy()
        assert np.isfinite(a).all()
        assert np.abs(a - b).max() <= TOL * np.abs(b).max()


def test_noalloc_rejects_sizes_beyond_its_scratch():
    t = (1 << 19) // 3 + 1  # t * dim exceeds the 2^19-double scratch
    tg = torch.zeros(t, 3, dtype=torch.float64, device=DEV)
    idx = torch.zeros(t, dtype=torch.int64, device=DEV)
    src = torch.zeros(8, 3, dtype=torch.float64, device=DEV)
    mass = torch.ones(8, dtype=torch.float64, device=DEV)
    out = torch.empty_like(tg)
    assert _call("augur_direct_sum_fp64_noalloc", tg, idx, src, mass, 3, 1e-3, out) == -34  # AUGUR_ERANGE
