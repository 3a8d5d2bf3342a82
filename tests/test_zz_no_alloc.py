"""tf_vec_mdot_noalloc: the multi-dot for callers that cannot allocate device
memory (for instance a host application that gives the library a fixed
device-memory budget, or a loop that must avoid the synchronisation of
cudaMalloc/cudaFree).  It must agree with the allocating tf_vec_mdot, on
consecutive calls that reuse its fixed scratch array, and reject sizes beyond
its limit of 64 vectors.  The file is named to be collected last."""

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

RTOL = 1e-13


def _call_both(lib, torch, n, k, seed):
    stream = torch.cuda.current_stream().cuda_stream
    rng = np.random.default_rng(seed)
    V = torch.as_tensor(rng.standard_normal((k, n))).cuda()
    w = torch.as_tensor(rng.standard_normal(n)).cuda()
    ref = torch.empty(k, dtype=torch.float64, device='cuda')
    wb = lib.tf_vec_mdot_workspace_bytes(n, k)
    work = torch.empty(wb // 8 + 1, dtype=torch.float64, device='cuda')
    assert lib.tf_vec_mdot(n, k, V.data_ptr(), n, w.data_ptr(), ref.data_ptr(), work.data_ptr(),
                           work.numel() * 8, stream) == 0
    out = torch.full((k,), np.nan, dtype=torch.float64, device='cuda')
    assert lib.tf_vec_mdot_noalloc(n, k, V.data_ptr(), n, w.data_ptr(), out.data_ptr(), stream) == 0
    torch.cuda.synchronize()
    return out.cpu().numpy(), ref.cpu().numpy(), (V.cpu().numpy() @ w.cpu().numpy())


def test_noalloc_mdot_matches_allocating_mdot_on_consecutive_calls():
    import torch
    from transiflow_gb300 import _lib
    lib = _lib.load()
    # the first call fills the whole scratch array, the second reuses it with
    # a smaller problem, so stale partial sums would show up as a mismatch
    for n, k, seed in ((300_007, 64, 1), (12_345, 5, 2)):
        out, ref, exact = _call_both(lib, torch, n, k, seed)
        scale = np.abs(exact).max()
        assert np.all(np.abs(out - ref) <= RTOL * scale)
        assert np.all(np.abs(out - exact) <= 1e-11 * scale)


def test_noalloc_mdot_rejects_sizes_beyond_its_limit():
    import torch
    from transiflow_gb300 import _lib
    lib = _lib.load()
    n, k = 1000, 65
    V = torch.zeros((k, n), dtype=torch.float64, device='cuda')
    w = torch.zeros(n, dtype=torch.float64, device='cuda')
    out = torch.zeros(k, dtype=torch.float64, device='cuda')
    rc = lib.tf_vec_mdot_noalloc(n, k, V.data_ptr(), n, w.data_ptr(), out.data_ptr(),
                                 torch.cuda.current_stream().cuda_stream)
    assert rc == 4   # TF_ERR_SIZE
    assert lib.tf_error_string(rc).decode() == 'size exceeds a compiled-in limit'
