"""rq_sort_pairs_noalloc: the radix sort for callers that must not allocate
device memory while they run (a serving loop held to a fixed memory budget,
code whose device memory belongs to another allocator, a latency-critical loop
where cudaMalloc/cudaFree would synchronize the device).  Its working memory
is a fixed array inside the library, shared by every call, so this test runs
two calls in a row and checks that the second is not disturbed by what the
first left behind.  It compares through the C ABI against rq_sort_pairs, the
existing entry point, bit for bit (integer work).

Collected last on purpose (file name) so that a run stopping at the first
failure has run everything else first; it also passes alone in a new process.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _sorted_by_existing_entry_point(engine, keys, vals, bits):
    k, v = engine.sort_pairs(keys.copy(), vals.copy(), key_bits=bits)
    return k, v


def test_noalloc_sort_matches_rq_sort_pairs_on_two_calls_in_a_row(engine, rqm):
    import torch
    stream = torch.cuda.current_stream()
    # Key widths of 4, 1 and 3 digit passes: after an odd number of passes the
    # result is copied back from the fixed array into the caller's buffers.
    # Each call is smaller than the one before, so stale contents of the
    # shared array would show.
    cases = [(rqm.SORT_NOALLOC_MAX_PAIRS, 30, 1), (100_003, 32, 2), (77_777, 7, 3), (50_001, 24, 4)]
    for n, bits, seed in cases:
        rng = np.random.default_rng(seed)
        keys = rng.integers(0, 1 << bits, n, dtype=np.uint64).astype(np.uint32)
        keys[::7] = keys[0]  # ties: stability matters
        vals = np.arange(n, dtype=np.uint32)
        want_k, want_v = _sorted_by_existing_entry_point(engine, keys, vals, bits)
        dk = torch.from_numpy(keys.view(np.int32).copy()).cuda()
        dv = torch.from_numpy(vals.view(np.int32).copy()).cuda()
        torch.cuda.synchronize()
        st = rqm.sort_pairs_noalloc(dk.data_ptr(), dv.data_ptr(), n, bits, stream.cuda_stream or None)
        assert st == 0, rqm.STATUS_NAMES.get(st, st)
        got_k = dk.cpu().numpy().view(np.uint32)
        got_v = dv.cpu().numpy().view(np.uint32)
        assert np.array_equal(got_k, want_k)
        assert np.array_equal(got_v, want_v)


def test_noalloc_sort_rejects_sizes_beyond_its_array(rqm):
    import torch
    n = rqm.SORT_NOALLOC_MAX_PAIRS + 1
    dk = torch.zeros(n, dtype=torch.int32, device="cuda")
    dv = torch.zeros(n, dtype=torch.int32, device="cuda")
    assert rqm.sort_pairs_noalloc(dk.data_ptr(), dv.data_ptr(), n, 32, None) == 1  # INVALID_ARGUMENT


def test_noalloc_sort_single_pair_is_left_unchanged(rqm):
    import torch
    dk = torch.tensor([123456789], dtype=torch.int32, device="cuda")
    dv = torch.tensor([42], dtype=torch.int32, device="cuda")
    assert rqm.sort_pairs_noalloc(dk.data_ptr(), dv.data_ptr(), 1, 32, None) == 0
    assert int(dk.item()) == 123456789 and int(dv.item()) == 42
