"""The allocation-free sigma entry point (qdkgb_sigma_split_noalloc).

It serves callers that cannot allocate device memory while they run (inside a
CUDA graph capture, under another allocator's pool): inputs, outputs and the
stream are theirs, the scratch is a fixed device array inside the library.  Here
it is called through the C ABI on device arrays the test owns and compared with
the context-based full-precision sigma (qdkgb_spmv, FP64 mode on the same split
storage) and with the oracle's CSR sigma, on two calls in a row, at the
tolerance of the other sigma tests (1e-12 relative).  The size check, which
needs no GPU, is tested in test_capi_cpu.py.  This file is collected last on
purpose.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _split(values):
    hi = values.astype(np.float32)
    lo = (values - hi.astype(np.float64)).astype(np.float32)
    return hi, lo


def test_noalloc_sigma_matches_context_sigma(pkg, oracle):
    import torch

    pkg.build.build()
    capi = pkg.capi
    T, V, _ = pkg.integrals.synthetic_integrals(8, 16, seed=31)
    a, b = pkg.determinants.fci_space(8, 4, 4)
    n = len(a)
    with capi.Context(0) as ctx:
        ctx.set_integrals(T, V)
        ctx.set_dets(a, b)
        ctx.build_hamiltonian(storage=capi.H_SPLIT32)
        rp, ci, nz = ctx.get_csr(64)
        hi, lo = _split(nz)
        dev = torch.device("cuda:0")
        d_rp = torch.from_numpy(rp).to(dev)
        d_ci = torch.from_numpy(ci.astype(np.int32)).to(dev)
        d_hi = torch.from_numpy(hi).to(dev)
        d_lo = torch.from_numpy(lo).to(dev)
        stream = torch.cuda.Stream()
        M = oracle.build_csr(oracle.Hamiltonian(T, V), a, b)
        rng = np.random.default_rng(5)
        for call in range(2):
            x = rng.normal(size=n)
            ref = ctx.spmv(x, capi.PREC_FP64)
            d_x = torch.from_numpy(x).to(dev)
            d_y = torch.full((n,), float("nan"), dtype=torch.float64, device=dev)
            torch.cuda.synchronize()
            capi.sigma_split_noalloc(n, d_rp.data_ptr(), d_ci.data_ptr(), d_hi.data_ptr(), d_lo.data_ptr(),
                                     d_x.data_ptr(), d_y.data_ptr(), stream.cuda_stream)
            stream.synchronize()
            y = d_y.cpu().numpy()
            assert np.all(np.isfinite(y)), call
            assert np.max(np.abs(y - ref)) <= 1e-12 * np.max(np.abs(ref)), call
            yo = M.spmv(x)
            assert np.max(np.abs(y - yo)) <= 1e-12 * np.max(np.abs(yo)), call
