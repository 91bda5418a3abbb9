"""mf_vegas_accumulate_noalloc: the VEGAS accumulation for callers that cannot
allocate device memory (its scratch is a fixed array inside the library).
Called through the C ABI and compared with mf_vegas_accumulate on the same
inputs, twice in a row (the second call reuses the array the first left
behind).  This file runs last so that a failure here leaves every other test
already run."""

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _inputs(torch, seed, N, ndim, nb):
    rng = np.random.default_rng(seed)
    f = torch.tensor(rng.exponential(size=N), device="cuda")
    jac = torch.tensor(rng.uniform(0.5, 2.0, size=N), device="cuda")
    bins = torch.tensor(rng.integers(0, nb, size=(ndim, N)).astype(np.int32), device="cuda")
    return f, jac, bins


def test_noalloc_accumulate_matches_allocating(cuda):
    import torch

    from madflow_gb300 import _lib

    lib = _lib.load()
    assert hasattr(lib, "mf_vegas_accumulate_noalloc")
    ndim, nb = 18, 50
    for call, (seed, N) in enumerate(((1, 100_000), (2, 37_777))):
        f, jac, bins = _inputs(torch, seed, N, ndim, nb)
        ref = torch.empty(2 + ndim * nb, dtype=torch.float64, device="cuda")
        out = torch.full_like(ref, float("nan"))
        _lib.call("mf_vegas_accumulate", f.data_ptr(), jac.data_ptr(), bins.data_ptr(), N, ndim, nb, 1.0 / N,
                  ref.data_ptr(), None)
        _lib.call("mf_vegas_accumulate_noalloc", f.data_ptr(), jac.data_ptr(), bins.data_ptr(), N, ndim, nb, 1.0 / N,
                  out.data_ptr(), None)
        torch.cuda.synchronize()
        r, o = ref.cpu().numpy(), out.cpu().numpy()
        assert np.all(np.isfinite(o)), call
        # same kernels, same block count, fixed summation order: bit-identical
        np.testing.assert_array_equal(o, r)


def test_noalloc_rejects_oversize(cuda):
    import torch

    from madflow_gb300 import _lib

    lib = _lib.load()
    f, jac, bins = _inputs(torch, 3, 1000, 41, 50)  # 41 * 50 = 2050 bins > 2048
    res = torch.empty(2 + 41 * 50, dtype=torch.float64, device="cuda")
    st = lib.mf_vegas_accumulate_noalloc(f.data_ptr(), jac.data_ptr(), bins.data_ptr(), 1000, 41, 50, 1e-3,
                                         res.data_ptr(), None)
    assert st == _lib.MF_ERR_CAPACITY
