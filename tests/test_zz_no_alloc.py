"""laml_inside_noalloc: the inside pass for callers that may not allocate
device memory (a host runtime owning the memory budget, or a loop that cannot
take the synchronisation of cudaMalloc/cudaFree).  Called through the C ABI;
its per-tree log-likelihoods must equal laml_inside's on two calls in a row.
This file sorts last so a failure here never hides the other tests."""
import ctypes as C

import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

from laml_gb300 import _native as N  # noqa: E402
from laml_gb300 import problem as PB  # noqa: E402
from laml_gb300 import synth  # noqa: E402


def test_inside_noalloc_matches_inside_twice():
    w = synth.pmm_workload(200, 30, 4, 20, 0.5, 0.1, 0.15, seed=77, n_trees=6, nni=True)
    b = PB.make_batch(w.newicks, w.rows, w.Q, w.leaf_order, compat=True, nu=0.1, phi=0.15)
    b.branch_terms()
    b.inside(update_em=False)
    torch.cuda.synchronize()
    ref = b.work["tr_llh"].cpu().numpy().copy()
    ref_site = [b.site_llh(t) for t in range(b.T)]   # real sites only (not the padding)
    lib = N.lib()
    # the caller's batch without partial buffers: the entry point brings its own
    nb = N.Batch()
    C.pointer(nb)[0] = b.b
    nb.in_part = None
    nb.in_x = None
    nb.in_h = None
    nb.in_dot = None
    stream = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    for _ in range(2):
        b.work["tr_llh"].fill_(float("nan"))
        b.work["llh_site"].fill_(float("nan"))
        rc = lib.laml_inside_noalloc(C.byref(nb), b.sizes["part_floats"], b.sizes["scalar_len"],
                                     stream)
        assert rc == 0, lib.laml_last_error()
        torch.cuda.synchronize()
        got = b.work["tr_llh"].cpu().numpy()
        np.testing.assert_allclose(got, ref, rtol=1e-6)
        for t in range(b.T):
            np.testing.assert_allclose(b.site_llh(t), ref_site[t], rtol=1e-6)


def test_inside_noalloc_rejects_oversized_batches():
    w = synth.pmm_workload(40, 10, 3, 8, 0.5, 0.1, 0.15, seed=78)
    b = PB.make_batch(w.newicks, w.rows, w.Q, w.leaf_order, compat=True)
    lib = N.lib()
    rc = lib.laml_inside_noalloc(C.byref(b.b), 1 << 30, b.sizes["scalar_len"],
                                 C.c_void_p(torch.cuda.current_stream().cuda_stream))
    assert rc == N.LAML_OK - 1   # LAML_ERR_ARG
    assert b"fixed scratch" in lib.laml_last_error()
    # sizes below the batch's own plan are refused before any launch (the
    # level kernels write at the plan's offsets)
    rc = lib.laml_inside_noalloc(C.byref(b.b), b.sizes["part_floats"] - 8, b.sizes["scalar_len"],
                                 C.c_void_p(torch.cuda.current_stream().cuda_stream))
    assert rc == N.LAML_OK - 1
    assert b"plan sizes" in lib.laml_last_error()
