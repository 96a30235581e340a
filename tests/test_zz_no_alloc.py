"""rrea_gpu_order_secondaries_noalloc (the allocation-free ordering pass,
called through the C-ABI) against the ordering inside the existing entry
point rrea_gpu_apply_electrons.

The pass only moves records, so the tolerance is exact equality of the
112-byte records.  Two calls run back to back on the same device scratch
with different sizes, into output buffers filled with 0xFF first, to show
that nothing needs to be cleared between calls.  This file sorts last so it
also runs after every other GPU test in the same process."""
import numpy as np
import pytest

from conftest import TABLES

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def env():
    torch = pytest.importorskip("torch")
    from rrea_feedback_warpx_amrex_geant4_gb300 import build, gpu, workloads
    build.build()
    cfg = workloads.make_config(gpu, "scaleup_c1")
    ctx = gpu.RreaGpuContext(cfg, 8192)
    ctx.load_tables(TABLES)
    ctx.set_field(**workloads.make_field("scaleup_c1"))
    yield torch, gpu, workloads, ctx
    ctx.close()


def _device(torch, host):
    return torch.from_numpy(np.ascontiguousarray(host).view(np.uint8).copy()).cuda()


def _order(torch, gpu, counts, unordered, n_parents, fill=255):
    d_counts = _device(torch, counts.astype(np.uint32))
    d_in = _device(torch, unordered)
    d_out = torch.full_like(d_in, fill)
    torch.cuda.synchronize()
    status, msg = gpu.order_secondaries_noalloc(d_counts.data_ptr(), n_parents, d_in.data_ptr(), len(unordered),
                                                d_out.data_ptr(), torch.cuda.current_stream().cuda_stream)
    out = d_out.cpu().numpy().view(gpu.SECONDARY_DTYPE)
    return status, msg, out


@pytest.mark.parametrize("n,seed,step", [(4096, 31, 2), (1500, 37, 9)])
def test_noalloc_ordering_matches_apply_electrons(env, n, seed, step):
    torch, gpu, workloads, ctx = env
    arr = workloads.make_electrons("scaleup_c1", n, seed=seed)
    ref = ctx.apply_electrons(arr, step, 5.0e-10)       # ordered by the existing entry point
    assert len(ref) > 0
    counts = np.bincount(ref["parent_index"], minlength=n)
    for call in range(2):                                # two calls in a row, shuffled differently
        perm = np.random.default_rng(seed * 10 + call).permutation(len(ref))
        status, msg, out = _order(torch, gpu, counts, ref[perm], n)
        assert status == 0, msg
        assert out.tobytes() == ref.tobytes()


def test_noalloc_rejects_more_parents_than_its_scratch(env):
    torch, gpu, workloads, ctx = env
    n = gpu.NOALLOC_MAX_PARENTS + 1
    status, msg = gpu.order_secondaries_noalloc(0, n, 0, 0, 0, None)
    assert status == 8, msg                              # RREA_GPU_ERR_CAPACITY
    assert str(gpu.NOALLOC_MAX_PARENTS) in msg


def test_noalloc_flags_inconsistent_records(env):
    torch, gpu, workloads, ctx = env
    arr = workloads.make_electrons("scaleup_c1", 512, seed=41)
    ref = ctx.apply_electrons(arr, 1, 5.0e-10)
    assert len(ref) > 1
    counts = np.bincount(ref["parent_index"], minlength=512)
    bad = ref.copy()
    bad["lineage"][0] = counts[bad["parent_index"][0]]   # one past its parent's count
    status, msg, out = _order(torch, gpu, counts, bad, 512)
    assert status == 9, msg                              # RREA_GPU_ERR_INVALID_STATE
    assert "lineage" in msg
    # the pass stays usable: a consistent call right after succeeds
    status, msg, out = _order(torch, gpu, counts, ref[::-1].copy(), 512)
    assert status == 0, msg
    assert out.tobytes() == ref.tobytes()


def test_noalloc_at_its_maximum_parent_count(env):
    """n_parents = RREA_GPU_NOALLOC_MAX_PARENTS exactly: the scan's last
    block sums and the error word sit at the far end of the fixed array.
    Counts mostly zero, a few thousand records; the expected order is a NumPy
    reordering by (parent_index, lineage)."""
    torch, gpu, workloads, ctx = env
    n = gpu.NOALLOC_MAX_PARENTS
    rng = np.random.default_rng(2718)
    counts = np.zeros(n, dtype=np.int64)
    parents = rng.choice(n, size=1500, replace=False)
    parents[:2] = (0, n - 1)                             # both ends of the parent range
    counts[parents] = rng.integers(1, 5, size=parents.size)
    recs = np.zeros(int(counts.sum()), dtype=gpu.SECONDARY_DTYPE)
    recs["parent_index"] = np.repeat(np.arange(n), counts)
    starts = np.cumsum(counts) - counts
    recs["lineage"] = np.arange(len(recs)) - np.repeat(starts, counts)
    recs["energy_eV"] = rng.uniform(1.0, 2.0, len(recs))
    recs["species"] = rng.integers(0, 3, len(recs))
    expected = recs.copy()                               # already in (parent, lineage) order
    for call in range(2):
        perm = np.random.default_rng(call).permutation(len(recs))
        status, msg, out = _order(torch, gpu, counts, recs[perm], n)
        assert status == 0, msg
        assert out.tobytes() == expected.tobytes()


def test_noalloc_flags_a_duplicated_pair(env):
    """One record duplicated in place of another: the counts still sum to
    n_secondaries and every lineage is in range, yet one output slot would
    stay unwritten.  The call reports it instead of returning OK."""
    torch, gpu, workloads, ctx = env
    arr = workloads.make_electrons("scaleup_c1", 512, seed=43)
    ref = ctx.apply_electrons(arr, 1, 5.0e-10)
    assert len(ref) > 2
    counts = np.bincount(ref["parent_index"], minlength=512)
    dup = ref.copy()
    dup[1] = dup[0]                                      # record 1 lost, record 0 twice
    status, msg, out = _order(torch, gpu, counts, dup, 512)
    assert status == 9, msg                              # RREA_GPU_ERR_INVALID_STATE
    assert "share" in msg
    status, msg, out = _order(torch, gpu, counts, ref, 512)
    assert status == 0, msg
    assert out.tobytes() == ref.tobytes()
