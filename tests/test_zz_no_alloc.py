"""The allocation-free sort entry point (sad_radix_sort_pairs_noalloc), called through the
C ABI, against the entry point that takes caller scratch (sad_radix_sort_pairs) on the same
inputs.  The sort is integer work, so the results must be identical; two calls in a row
exercise the reuse of the library's fixed scratch.  This file is collected last so the
entry point also runs after every other test in the same process."""
import ctypes as C

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

MAX_PAIRS = 262144  # SAD_NOALLOC_SORT_MAX_PAIRS


def _ptr(t):
    return C.c_void_p(t.data_ptr())


def _sort_with_scratch(lib, pairs, max_key):
    n = pairs.shape[0]
    out = pairs.clone()
    temp = torch.empty(max(16, lib.sad_radix_sort_temp_bytes(n)), dtype=torch.uint8, device="cuda")
    st = lib.sad_radix_sort_pairs(_ptr(out), n, max_key, _ptr(temp), temp.numel(), None)
    assert st == 0, lib.sad_last_error().decode()
    return out


def _sort_noalloc(lib, pairs, max_key):
    out = pairs.clone()
    st = lib.sad_radix_sort_pairs_noalloc(_ptr(out), pairs.shape[0], max_key, None)
    assert st == 0, lib.sad_last_error().decode()
    return out


def _pairs(n, max_key, seed):
    rng = np.random.default_rng(seed)
    keys = rng.integers(0, max_key, n, dtype=np.uint64).astype(np.uint32)
    vals = np.arange(n, dtype=np.uint32)
    a = np.stack([keys, vals], axis=1)
    return torch.from_numpy(a.view(np.int32)).cuda()


@pytest.fixture(scope="module")
def lib(cuda):
    from sad_gb300 import _lib
    return _lib.load()


@pytest.mark.parametrize("n,max_key", [(200003, 0xFFFFFFFF), (MAX_PAIRS, 65536), (4097, 1000)])
def test_noalloc_sort_matches_scratch_entry_point(lib, n, max_key):
    pairs = _pairs(n, max_key, n)
    want = _sort_with_scratch(lib, pairs, max_key)
    for _ in range(2):  # two calls in a row reuse the fixed scratch
        got = _sort_noalloc(lib, pairs, max_key)
        torch.cuda.synchronize()
        assert torch.equal(got, want)
    keys = want[:, 0].cpu().numpy().view(np.uint32)
    assert np.all(keys[1:] >= keys[:-1])


def test_noalloc_sort_rejects_oversize_and_handles_trivial(lib):
    big = torch.zeros((MAX_PAIRS + 1, 2), dtype=torch.int32, device="cuda")
    st = lib.sad_radix_sort_pairs_noalloc(_ptr(big), MAX_PAIRS + 1, 0xFFFFFFFF, None)
    assert st != 0
    assert b"SAD_NOALLOC_SORT_MAX_PAIRS" in lib.sad_last_error()
    one = torch.tensor([[7, 3]], dtype=torch.int32, device="cuda")
    assert lib.sad_radix_sort_pairs_noalloc(_ptr(one), 1, 100, None) == 0
    assert lib.sad_radix_sort_pairs_noalloc(None, 0, 100, None) == 0
    torch.cuda.synchronize()
    assert one.tolist() == [[7, 3]]


def test_noalloc_sort_on_a_side_stream_after_the_default_stream(lib):
    """The documented serialised use across streams: a call on the default stream, then,
    ordered after it by an event, a call on another stream; both results must equal the
    scratch-taking entry point's."""
    a = _pairs(150001, 0xFFFFFFFF, 11)
    b = _pairs(70001, 65536, 12)
    want_a = _sort_with_scratch(lib, a, 0xFFFFFFFF)
    want_b = _sort_with_scratch(lib, b, 65536)
    torch.cuda.synchronize()
    got_a = a.clone()
    got_b = b.clone()
    side = torch.cuda.Stream()
    done = torch.cuda.Event()
    st = lib.sad_radix_sort_pairs_noalloc(_ptr(got_a), a.shape[0], 0xFFFFFFFF, None)
    assert st == 0, lib.sad_last_error().decode()
    done.record(torch.cuda.default_stream())
    side.wait_event(done)
    st = lib.sad_radix_sort_pairs_noalloc(_ptr(got_b), b.shape[0], 65536, C.c_void_p(side.cuda_stream))
    assert st == 0, lib.sad_last_error().decode()
    side.synchronize()
    torch.cuda.synchronize()
    assert torch.equal(got_a, want_a)
    assert torch.equal(got_b, want_b)
