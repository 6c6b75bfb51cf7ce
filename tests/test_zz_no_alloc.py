"""The allocation-free lookup entry point (openmc_gb300_xs_lookup_noalloc).

Some callers cannot allocate device memory while they call into the library:
an embedding code that runs under a fixed memory budget or inside a memory
pool it does not own.  For them the library offers one lookup entry point whose
sort scratch is a static device array instead of memory allocated on demand.
This test checks, through the C ABI, that two calls in a row return exactly
what the allocating entry point returns for the same lookups, and that a
request larger than the static scratch is refused with an error.  It runs last
so that a failure here comes after every other test has run.
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
    tables.lookup_device(n, d_mat.data_ptr(), d_e.data_ptr(), ref.data_ptr(), ref_hash.data_ptr(), sort=True)
    torch.cuda.synchronize()
    stream = torch.cuda.current_stream().cuda_stream
    scale = ref.abs().max().item()
    for _ in range(2):
        out = torch.full((n, 5), float("nan"), dtype=torch.float64, device=dev)
        h = torch.full((n,), -1, dtype=torch.int32, device=dev)
        tables.lookup_noalloc(n, d_mat.data_ptr(), d_e.data_ptr(), out.data_ptr(), h.data_ptr(), stream=stream)
        torch.cuda.synchronize()
        assert torch.equal(h, ref_hash)
        # same tolerance as the FP64 lookup parity test (1e-12 relative)
        assert torch.allclose(out, ref, rtol=1e-12, atol=1e-12 * scale)
    with pytest.raises(lib.InvalidArgumentError):
        tables.lookup_noalloc(1 << 23, d_mat.data_ptr(), d_e.data_ptr(), ref.data_ptr(), None, stream=stream)
    tables.close()
