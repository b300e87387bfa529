"""The allocation-free entry point regot_erot_dual_obj_grad_noalloc.

It serves callers that cannot allocate device memory (inside another
framework's CUDA-graph capture or custom call, or in loops that cannot
afford cudaMalloc's synchronisation): its scratch is a fixed static device
array. This test calls it through the C ABI with device buffers that the
test allocates, twice in a row on the same scratch, and checks each result
against the allocating entry point regot_erot_dual_obj_grad and against the
FP64 oracle on the same FP32-rounded M, within the mixed-precision
tolerance of the other parity tests. A GPU-side failure (a bounded wait of
the dense pass that gives up, forced by a wait limit of 0) shows as NaN in
the outputs, since the call returns before the GPU runs it. The file name
makes pytest collect it last.
"""
import ctypes as C

import numpy as np
import pytest

from problems import erot_points

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")
regot = pytest.importorskip("regot")

import regot_oracle as O

# Mixed precision (FP32 M and exp2, FP64 duals): the objective and the row
# and column sums of T agree with the FP64 evaluation on the same FP32 M to
# ~1e-7 relative. The duals here are random, so the sums are O(100) and the
# gradient is compared relative to its own largest entry.
TOL = 1e-6


def _call(M_dev, n, m, gamma, a_dev, b_dev, reg):
    from regot import _lib

    lib = _lib.load()
    g_dev = torch.from_numpy(np.ascontiguousarray(gamma)).cuda()
    grad = torch.empty(n + m - 1, dtype=torch.float64, device="cuda")
    obj = torch.empty(1, dtype=torch.float64, device="cuda")
    stream = torch.cuda.current_stream().cuda_stream
    rc = lib.regot_erot_dual_obj_grad_noalloc(
        C.c_void_p(M_dev.data_ptr()), M_dev.stride(0), n, m, C.c_void_p(g_dev.data_ptr()),
        C.c_void_p(a_dev.data_ptr()), C.c_void_p(b_dev.data_ptr()), float(reg),
        C.c_void_p(grad.data_ptr()), C.c_void_p(obj.data_ptr()), C.c_void_p(stream))
    torch.cuda.synchronize()
    return rc, float(obj.item()), grad.cpu().numpy()


def test_noalloc_matches_allocating_entry_point_twice():
    n, m, reg = 300, 260, 0.05
    M, a, b = erot_points(n, m, seed=7, dtype=np.float32)
    P = regot.Problem(M, a, b, precision="mixed")
    M_dev = torch.from_numpy(M).cuda()
    a_dev = torch.from_numpy(a).cuda()
    b_dev = torch.from_numpy(b).cuda()
    rng = np.random.default_rng(3)
    for call in range(2):
        gamma = rng.standard_normal(n + m - 1) * 0.02
        rc, f_new, g_new = _call(M_dev, n, m, gamma, a_dev, b_dev, reg)
        assert rc == 0, f"call {call}: status {rc}"
        f_ref, g_ref = P.erot_dual_obj_grad(reg, gamma)
        assert abs(f_new - f_ref) <= TOL * max(1.0, abs(f_ref)), call
        np.testing.assert_allclose(g_new, g_ref, rtol=0, atol=TOL * np.abs(g_ref).max())
        f_o, g_o = O.erot_dual_obj_grad(M.astype(np.float64), a, b, reg, gamma)
        assert abs(f_new - f_o) <= TOL * max(1.0, abs(f_o)), call
        np.testing.assert_allclose(g_new, g_o, rtol=0, atol=TOL * np.abs(g_o).max())
    P.close()


def test_noalloc_reports_a_wait_that_gave_up_as_nan():
    from regot import _lib

    lib = _lib.load()
    n, m, reg = 300, 260, 0.05
    M, a, b = erot_points(n, m, seed=7, dtype=np.float32)
    M_dev = torch.from_numpy(M).cuda()
    a_dev = torch.from_numpy(a).cuda()
    b_dev = torch.from_numpy(b).cuda()
    gamma = np.random.default_rng(5).standard_normal(n + m - 1) * 0.02
    old = lib.regot_set_wait_limit(0)
    try:
        rc, f, g = _call(M_dev, n, m, gamma, a_dev, b_dev, reg)
    finally:
        lib.regot_set_wait_limit(old)
    assert rc == 0
    assert np.isnan(f) and np.isnan(g).all()
    # the error word is cleared by the next call
    rc, f, g = _call(M_dev, n, m, gamma, a_dev, b_dev, reg)
    f_o, g_o = O.erot_dual_obj_grad(M.astype(np.float64), a, b, reg, gamma)
    assert rc == 0 and np.isfinite(f) and np.isfinite(g).all()
    assert abs(f - f_o) <= TOL * max(1.0, abs(f_o))


def test_noalloc_rejects_problems_beyond_the_scratch():
    from regot import _lib

    n = m = 20000  # needs more than the 16 MiB scratch
    M_dev = torch.zeros((n, m), dtype=torch.float32, device="cuda")
    v = torch.ones(n + m, dtype=torch.float64, device="cuda")
    rc, _, _ = _call(M_dev, n, m, np.zeros(n + m - 1), v[:n], v[:m], 0.1)
    assert rc == _lib.REGOT_ERR_TOO_LARGE
