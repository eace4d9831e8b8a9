"""The allocation-free line solver against the allocating one.

hamstr_gpu_block_tridag4_noalloc exists for callers that cannot allocate
device memory on every call (loops beside work on other streams, where the
allocating call's cudaFree would wait for the whole device, and hosts whose
device memory belongs to their own pool).  It runs the same kernel with a
fixed scratch array inside the library, so its results must equal the
allocating entry point's bit for bit, on consecutive calls that reuse the
shared scratch.  This file is collected last on purpose.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _systems(rng, nlines, n):
    import torch
    a = rng.standard_normal((nlines, n, 4, 4))
    b = rng.standard_normal((nlines, n, 4, 4)) + 6.0 * np.eye(4)
    c = rng.standard_normal((nlines, n, 4, 4))
    f = rng.standard_normal((nlines, n, 4))
    return [torch.from_numpy(x).cuda() for x in (a, b, c, f)]


@pytest.mark.parametrize("periodic", [False, True])
def test_noalloc_equals_allocating_on_two_calls(native_lib, periodic):
    import torch
    from hamstr_oop_gb300 import native
    rng = np.random.default_rng(77 + int(periodic))
    for nlines, n in ((16, 48), (40, 129)):          # second call reuses the scratch
        A, B, C, F = _systems(rng, nlines, n)
        want = F.clone()
        native.block_tridag4(A, B, C, want, periodic)
        got = F.clone()
        native.block_tridag4_noalloc(A, B, C, got, periodic)
        torch.cuda.synchronize()
        assert torch.equal(got, want), "no-alloc solve differs (periodic=%s, %dx%d)" % (periodic, nlines, n)


def test_noalloc_rejects_oversize(native_lib):
    import torch
    from hamstr_oop_gb300 import native
    n = 1024
    nlines = (1 << 20) // (80 * n + 16) + 1
    z = torch.zeros((nlines, n, 4, 4), dtype=torch.float64, device="cuda")
    f = torch.zeros((nlines, n, 4), dtype=torch.float64, device="cuda")
    with pytest.raises(native.HamstrError) as ei:
        native.block_tridag4_noalloc(z, z, z, f, False)
    assert ei.value.status == -1 and "exceeds" in str(ei.value)
