"""rpgo_max_clique_heu_dev_noalloc (fixed device scratch, no allocation) gives
the same clique as rpgo_max_clique_heu_dev, on consecutive calls that share
the scratch array. Both are called through the C ABI with device adjacency.

Collected last on purpose: it must pass in a fresh process (the first call
does the per-device set-up) and after every other test.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _adjacency(n, words, seed, planted):
    """Bit-packed symmetric adjacency (n rows of `words` uint32): a planted
    clique of `planted` vertices plus random edges."""
    rng = np.random.default_rng(seed)
    dense = np.triu(rng.random((n, n)) < 0.05, 1)
    members = rng.choice(n, planted, replace=False)
    dense[np.ix_(members, members)] = True
    dense = np.triu(dense, 1)
    dense = dense | dense.T
    bits = np.zeros((n, words * 32), dtype=np.uint8)
    bits[:, :n] = dense
    packed = np.packbits(bits.reshape(n, words, 32)[:, :, ::-1], axis=2, bitorder="big")
    return packed.view(">u4").astype(np.uint32).reshape(n, words)


def _call(fn, adj_dev, n, words, first, seed, stream):
    out = np.full(max(n, 1), -7, dtype=np.int32)
    size = np.zeros(1, dtype=np.int32)
    rc = fn(n, C.c_void_p(adj_dev.data_ptr()), words, first, seed, out.ctypes.data_as(C.c_void_p),
            size.ctypes.data_as(C.c_void_p), C.c_void_p(stream))
    return rc, int(size[0]), out[: max(int(size[0]), 0)].copy()


def test_noalloc_clique_matches_existing_entry_point_on_consecutive_calls():
    import torch

    from rpgo_gb300 import capi

    lib = capi.load()
    dev = torch.device("cuda:0")
    stream = torch.cuda.current_stream(dev).cuda_stream
    cases = [
        # (n, words, seed, planted, first, seed_size): the second call is
        # smaller, with a padded row stride and an incremental seed, so that
        # anything left in the scratch by the first call would show.
        (3000, 94, 11, 150, 0, -1),
        (700, 40, 12, 60, 700 // 3, 5),
    ]
    for n, words, seed, planted, first, seed_size in cases:
        adj = torch.from_numpy(_adjacency(n, words, seed, planted).view(np.int32)).to(dev)
        torch.cuda.synchronize()
        allocs_ref = capi.buffer_alloc_count()
        rc_ref, size_ref, clique_ref = _call(lib.rpgo_max_clique_heu_dev, adj, n, words, first, seed_size, stream)
        # the counter sees the allocating entry point's buffers
        assert capi.buffer_alloc_count() > allocs_ref
        launches = capi.kernel_launch_count()
        allocs = capi.buffer_alloc_count()
        rc, size, clique = _call(lib.rpgo_max_clique_heu_dev_noalloc, adj, n, words, first, seed_size, stream)
        assert rc_ref == capi.OK and rc == capi.OK
        assert capi.kernel_launch_count() > launches
        # the promise itself: no device or pinned buffer was allocated
        assert capi.buffer_alloc_count() == allocs
        assert size == size_ref >= planted
        assert np.array_equal(clique, clique_ref)


def test_noalloc_clique_rejects_sizes_beyond_its_scratch():
    import torch

    from rpgo_gb300 import capi

    lib = capi.load()
    adj = torch.zeros(4, dtype=torch.int32, device="cuda:0")
    n = capi.CLIQUE_NOALLOC_MAX_N + 1
    rc, _, _ = _call(lib.rpgo_max_clique_heu_dev_noalloc, adj, n, (n + 31) // 32, 0, -1, 0)
    assert rc == capi.ERR_SIZE
    rc, _, _ = _call(lib.rpgo_max_clique_heu_dev_noalloc, adj, 64, capi.CLIQUE_NOALLOC_MAX_WORDS + 1, 0, -1, 0)
    assert rc == capi.ERR_SIZE
