"""mf_integrand_rows: the integrand on points in rows (madflow's xrand[N,
ndim]), read from device memory or straight from page-locked host memory
(zero-copy), with f written to either; the same values as mf_integrand on
the transposed points."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("prec", [0, 1])
def test_rows_equal_columns_and_host_memory(cuda, prec):
    torch = cuda
    from madflow_gb300 import _lib
    from madflow_gb300.vegas import FusedIntegrand

    integ = FusedIntegrand(4, kind=1, sqrts=13000.0, ptmin=60.0, etamax=2.5, drmin=0.4, precision=prec)
    N = 20_000
    x = torch.rand((N, integ.n_dim), dtype=torch.float64, device="cuda",
                   generator=torch.Generator(device="cuda").manual_seed(21))
    # mf_integrand on [ndim][N]
    f_cols = torch.empty(N, dtype=torch.float64, device="cuda")
    _lib.call("mf_integrand", integ.matrix.handle, ctypes.byref(integ._cs), x.T.contiguous().data_ptr(), N,
              f_cols.data_ptr(), None)
    f_dev = integ(x)  # rows, device memory
    x_host = x.cpu().pin_memory()
    f_host = torch.empty(N, dtype=torch.float64).pin_memory()
    integ(x_host, out=f_host)  # rows, page-locked host memory in and out
    torch.cuda.synchronize()
    a = f_cols.cpu().numpy()
    np.testing.assert_array_equal(f_dev.cpu().numpy(), a)
    np.testing.assert_array_equal(f_host.numpy(), a)
    assert np.count_nonzero(a) > N // 4


def test_rows_reject_pageable_host_memory(cuda):
    torch = cuda
    from madflow_gb300 import _lib
    from madflow_gb300.vegas import FusedIntegrand

    integ = FusedIntegrand(2, kind=0, sqrts=1000.0, precision=0)
    x = np.random.default_rng(1).uniform(size=(100, integ.n_dim))
    f = torch.empty(100, dtype=torch.float64, device="cuda")
    st = _lib.load().mf_integrand_rows(integ.matrix.handle, ctypes.byref(integ._cs), x.ctypes.data, 100,
                                       f.data_ptr(), None)
    assert st == _lib.MF_ERR_ARG
    with pytest.raises(ValueError):
        integ(torch.rand((10, integ.n_dim), dtype=torch.float64, device="cuda"), out=torch.empty(10))
