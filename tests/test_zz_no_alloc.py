"""The allocation-free lookup entry point (openmc_gb300_xs_lookup_noalloc).

Some callers cannot allocate device memory while they call into the library:
an embedding code that runs under a fixed memory budget or inside a memory
pool it does not own.  For them the library offers one lookup entry point whose
sort scratch is a static device array instead of memory allocated on demand.
This test checks, through the C ABI, that two calls in a row return exactly
what the allocating entry point returns for the same lookups, that the
device's free memory does not change across calls, that a material index
out of range only turns its own lookup into NaN (the shared scratch is not
written out of bounds: the next call is still exact), and that requests
larger than the static scratch (lookups or materials) are refused with an
error.  It runs last so that a failure here comes after every other test has
run.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_noalloc_lookup_matches_allocating_entry_point(built):
    import torch
    from openmc_gb300 import data, lib
    d = data.make_xsbench(n_nuc=24, n_points=3000, seed=9, mat_counts=(60, 5, 4, 12, 9))
    mats, e = data.xsbench_lookups(d, 300_000, seed=4)
    n = len(e)
    tables = lib.XSTables(d, fp32=False, max_lookups=n)
    dev = torch.device("cuda", 0)
    d_mat = torch.from_numpy(mats).to(dev)
    d_e = torch.from_numpy(e).to(dev)
    ref = torch.empty((n, 5), dtype=torch.float64, device=dev)
    ref_hash = torch.empty(n, dtype=torch.int32, device=dev)
    torch.cuda.synchronize()
    tables.lookup_device(n, d_mat.data_ptr(), d_e.data_ptr(), ref.data_ptr(), ref_hash.data_ptr(), sort=True)
    torch.cuda.synchronize()
    stream = torch.cuda.current_stream().cuda_stream
    scale = ref.abs().max().item()
    outs = [torch.full((n, 5), float("nan"), dtype=torch.float64, device=dev) for _ in range(3)]
    hs = [torch.full((n,), -1, dtype=torch.int32, device=dev) for _ in range(3)]
    torch.cuda.synchronize()
    # the first call may load the library's kernels; the two after it run
    # back to back with no other device work between the free-memory readings
    tables.lookup_noalloc(n, d_mat.data_ptr(), d_e.data_ptr(), outs[0].data_ptr(), hs[0].data_ptr(),
                          stream=stream)
    torch.cuda.synchronize()
    free_before = torch.cuda.mem_get_info()[0]
    for k in (1, 2):
        tables.lookup_noalloc(n, d_mat.data_ptr(), d_e.data_ptr(), outs[k].data_ptr(), hs[k].data_ptr(),
                              stream=stream)
    torch.cuda.synchronize()
    free_after = torch.cuda.mem_get_info()[0]
    assert free_after == free_before
    for k in range(3):
        assert torch.equal(hs[k], ref_hash)
        # same tolerance as the FP64 lookup parity test (1e-12 relative)
        assert torch.allclose(outs[k], ref, rtol=1e-12, atol=1e-12 * scale)

    # out-of-range material indices: NaN for those lookups only
    bad = mats.copy()
    bad[[3, 17, n - 1]] = [-5, len(d.mat_prob), 1 << 30]
    d_bad = torch.from_numpy(bad).to(dev)
    out = torch.zeros((n, 5), dtype=torch.float64, device=dev)
    torch.cuda.synchronize()
    tables.lookup_noalloc(n, d_bad.data_ptr(), d_e.data_ptr(), out.data_ptr(), None, stream=stream)
    torch.cuda.synchronize()
    ok = torch.ones(n, dtype=torch.bool, device=dev)
    ok[[3, 17, n - 1]] = False
    assert torch.isnan(out[~ok]).all()
    assert torch.allclose(out[ok], ref[ok], rtol=1e-12, atol=1e-12 * scale)
    again = torch.zeros((n, 5), dtype=torch.float64, device=dev)
    torch.cuda.synchronize()
    tables.lookup_noalloc(n, d_mat.data_ptr(), d_e.data_ptr(), again.data_ptr(), None, stream=stream)
    torch.cuda.synchronize()
    assert torch.allclose(again, ref, rtol=1e-12, atol=1e-12 * scale)

    with pytest.raises(lib.InvalidArgumentError):
        tables.lookup_noalloc(1 << 23, d_mat.data_ptr(), d_e.data_ptr(), ref.data_ptr(), None, stream=stream)
    tables.close()

    # 65 materials need 65 x 64 sort keys, more than the static 4,096
    big = data.make_xsbench(n_nuc=4, n_points=200, seed=1, mat_counts=(2,) * 65)
    t65 = lib.XSTables(big, fp32=False, max_lookups=16)
    try:
        with pytest.raises(lib.InvalidArgumentError):
            t65.lookup_noalloc(8, d_mat.data_ptr(), d_e.data_ptr(), ref.data_ptr(), None, stream=stream)
    finally:
        t65.close()
