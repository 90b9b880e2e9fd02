"""p3d_pe_heating_vec_noalloc: the PE kernel with its scratch in a fixed
device array, for callers that cannot let the library allocate device
memory (an application that hands the library a fixed memory budget, an
allocator that owns every device byte, a caller that cannot take the
synchronisation of a cudaMalloc).  Every array argument is a device pointer.

Called through the C ABI and compared with p3d_pe_heating_vec_dev, the entry
point that stages the same data in the library's grow-only workspace, on two
calls in a row with different inputs (the scratch keeps the previous call's
contents, so the second call checks that nothing stale is read).  This file
runs last so a failure here cannot hide earlier ones.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _inputs(seed, n):
    rng = np.random.default_rng(seed)
    return [10 ** rng.uniform(-3, 5, n), 10 ** rng.uniform(1, 4.5, n),
            10 ** rng.uniform(-12, -3, n), 10 ** rng.uniform(1, 7, n),
            rng.uniform(0.01, 2.0, n), rng.uniform(-0.5, 3.0, n)]


def test_noalloc_matches_workspace_entry_point():
    import torch

    from prism3d_gb300 import _lib as L
    from prism3d_gb300.tables import DustTables
    assert torch.cuda.is_available()
    tb = DustTables()
    tab = torch.from_numpy(np.ascontiguousarray(tb.pe_table)).cuda()
    bins = [np.ascontiguousarray(a, dtype=np.float64) for a in
            (tb.bin_sigma_abs, tb.bin_dn_da_da, tb.bin_is_nano.astype(np.float64))]
    dbins = [torch.from_numpy(a).cuda() for a in bins]
    n = 300001
    for call, seed in enumerate((5, 6)):
        cells = [torch.from_numpy(a).cuda() for a in _inputs(seed, n)]
        # the second call uses another table (scaled) and E_g grid origin, so
        # condensed tables left over from the first call would show
        eg_min = tb.eg_min if call == 0 else tb.eg_min + 0.05
        tab_c = tab if call == 0 else tab * 1.7
        ref = torch.empty(n, dtype=torch.float64, device="cuda")
        out = torch.full((n,), np.nan, dtype=torch.float64, device="cuda")
        grid = (L.dptr(tab_c), tb.n_bins, tb.log_psi_min, tb.log_psi_step, tb.n_psi, eg_min,
                tb.eg_step, tb.n_Eg)
        tail = (n, *[L.dptr(c) for c in cells])
        stream = torch.cuda.current_stream().cuda_stream
        # the workspace entry point takes the bin vectors from the host ...
        L.call("p3d_pe_heating_vec_dev", *grid, *[L.dptr(a) for a in bins], *tail, L.dptr(ref),
               stream)
        torch.cuda.synchronize()
        # ... the no-allocation one from device memory
        L.call("p3d_pe_heating_vec_noalloc", *grid, *[L.dptr(a) for a in dbins], *tail,
               L.dptr(out), stream)
        torch.cuda.synchronize()
        r, o = ref.cpu().numpy(), out.cpu().numpy()
        assert np.all(np.isfinite(o))
        np.testing.assert_allclose(o, r, rtol=1e-12, atol=0)


def test_noalloc_rejects_oversized_tables():
    from prism3d_gb300 import _lib as L
    one = np.ones(4)
    rc = L.lib.p3d_pe_heating_vec_noalloc(
        L.dptr(one), 1, 0.0, 0.1, 100, 0.0, 0.1, 100, L.dptr(one), L.dptr(one), L.dptr(one), 1,
        *[L.dptr(one)] * 7, None)
    assert rc == -1
    assert "no-allocation limit" in L.lib.p3d_last_error().decode()
