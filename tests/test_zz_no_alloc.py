"""gbhf_eigen_solve_noalloc: the eigen-solve for callers that cannot allocate
device memory during the call (for example code inside another framework's
custom-call hook, where the framework owns every buffer).  The caller hands
in device buffers; the solver works in the library's static device array.

Checked through the C ABI against the allocating entry point gbhf_eigen_solve
and against LAPACK (numpy.linalg.eigh), on calls in a row (each call finds
the previous call's data in the shared array), including n = 1 and the
array's largest sizes (n = 255, 256).  This file sorts last so a
stop-at-first-failure run has already run every other test; it also passes on
its own in a fresh process.
"""
import ctypes as C

import numpy as np
import pytest

from gbhf import _lib

pytestmark = pytest.mark.gpu

TOL = 1e-12   # same eigenvalue tolerance as tests/test_gpu_linalg.py (relative to the spectrum's scale)


def _sym(n, seed):
    a = np.random.default_rng(seed).standard_normal((n, n))
    return a + a.T


def _solve_noalloc(lib, a, torch):
    n = a.shape[0]
    d_a = torch.from_numpy(np.ascontiguousarray(a)).to("cuda")
    d_w = torch.empty(n, dtype=torch.float64, device="cuda")
    d_v = torch.empty((n, n), dtype=torch.float64, device="cuda")
    stream = torch.cuda.current_stream().cuda_stream
    s = lib.gbhf_eigen_solve_noalloc(n, C.c_void_p(d_a.data_ptr()), C.c_void_p(d_w.data_ptr()),
                                     C.c_void_p(d_v.data_ptr()), C.c_void_p(stream))
    torch.cuda.synchronize()
    return s, d_w.cpu().numpy(), d_v.cpu().numpy()


def _check(a, w, v, w_ref, v_ref):
    scale = max(1.0, np.abs(w_ref).max())
    np.testing.assert_allclose(w, w_ref, rtol=0, atol=TOL * scale)
    # eigenvectors agree up to sign (the spectra here are non-degenerate)
    overlap = np.abs(np.sum(v * v_ref, axis=0))
    assert np.max(np.abs(overlap - 1.0)) < 1e-9
    assert np.max(np.abs(a @ v - v * w)) < 1e-11 * scale
    assert np.max(np.abs(v.T @ v - np.eye(a.shape[0]))) < 1e-12


def test_noalloc_eigen_solve_matches_allocating_entry_point(ctx):
    torch = pytest.importorskip("torch")
    assert torch.cuda.is_available()
    lib = _lib.load()
    # calls in a row with different sizes: the largest first, then smaller ones
    for call, (n, seed) in enumerate([(256, 10), (208, 11), (57, 12), (255, 13), (1, 14)]):
        a = _sym(n, seed)
        s, w, v = _solve_noalloc(lib, a, torch)
        assert s == 0, f"call {call}: status {_lib.STATUS.get(s, s)}"
        w_ctx, v_ctx = ctx.eigen_solve(a)           # the allocating entry point
        _check(a, w, v, w_ctx, v_ctx)
        w_np, v_np = np.linalg.eigh(a)              # LAPACK
        _check(a, w, v, w_np, v_np)


def test_noalloc_eigen_solve_rejects_sizes_beyond_its_array():
    torch = pytest.importorskip("torch")
    lib = _lib.load()
    n = 257
    assert n > 256
    buf = torch.zeros(8, dtype=torch.float64, device="cuda")
    p = C.c_void_p(buf.data_ptr())
    assert lib.gbhf_eigen_solve_noalloc(n, p, p, p, None) == 1   # GBHF_ERR_BAD_INPUT, nothing launched
    assert lib.gbhf_eigen_solve_noalloc(0, p, p, p, None) == 1
