"""sq_radix_sort_pairs_noalloc: the sort for callers that cannot allocate.

Some callers of this library cannot call cudaMalloc / cudaFree, for example a
host whose memory pool already owns the GPU's memory, or a loop that cannot
afford cudaFree's device-wide synchronisation.  The no-alloc entry point
serves them: they pass device buffers for the input and the output, and the
sort's scratch is a fixed array inside the library.  This file checks,
through the C ABI, that it returns exactly what the allocating entry point
(sq_radix_sort_pairs) returns, on two calls in a row (the scratch keeps the
previous call's contents), and that it rejects sizes beyond its fixed limit.
It sits in a file of its own, collected last.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

MAX_KEYS = 1 << 20
TOO_LARGE = 7


def noalloc_fn():
    import sequoia_gb300 as sq
    lib = sq.load_library()
    fn = lib.sq_radix_sort_pairs_noalloc
    fn.restype = C.c_int
    fn.argtypes = [C.c_void_p, C.c_void_p, C.c_uint32, C.c_uint32, C.c_uint32, C.c_void_p, C.c_void_p, C.c_void_p]
    return fn


def test_noalloc_sort_matches_allocating_sort(lib_built):
    torch = pytest.importorskip("torch")
    import sequoia_gb300 as sq
    ctx = sq.Context(0)
    fn = noalloc_fn()
    stream = torch.cuda.current_stream().cuda_stream
    # (n, key bits, digit bits): even and odd pass counts (4, 4, 6, 3, 1),
    # the largest size, a size one past a tile, a single key
    cases = [(300_001, 30, 8), (MAX_KEYS, 32, 10), (4097, 32, 6), (65_537, 24, 8), (1, 8, 8)]
    for n, key_bits, digit_bits in cases:
        for call in range(2):  # two calls in a row share the scratch
            rng = np.random.default_rng(1000 * call + n + digit_bits)
            keys = rng.integers(0, 1 << key_bits, n, dtype=np.uint64).astype(np.uint32)
            keys[: n // 4] = keys[0]  # duplicates: the order must be the stable one
            vals = rng.permutation(n).astype(np.uint32)
            want_k, want_v = ctx.radix_sort_pairs(keys, vals, key_bits, digit_bits)
            dk = torch.from_numpy(keys).cuda()
            dv = torch.from_numpy(vals).cuda()
            ok = torch.empty_like(dk)
            ov = torch.empty_like(dv)
            st = fn(dk.data_ptr(), dv.data_ptr(), n, key_bits, digit_bits, ok.data_ptr(), ov.data_ptr(), stream)
            assert st == 0, st
            assert np.array_equal(ok.cpu().numpy(), want_k), (n, key_bits, digit_bits, call)
            assert np.array_equal(ov.cpu().numpy(), want_v), (n, key_bits, digit_bits, call)
            # in place: the outputs may be the inputs
            st = fn(dk.data_ptr(), dv.data_ptr(), n, key_bits, digit_bits, dk.data_ptr(), dv.data_ptr(), stream)
            assert st == 0, st
            assert np.array_equal(dk.cpu().numpy(), want_k)
            assert np.array_equal(dv.cpu().numpy(), want_v)


def test_noalloc_rejects_oversize_and_host_pointers(lib_built):
    """Sizes beyond the fixed maximum are refused with SQ_ERR_TOO_LARGE.  The
    oversize request carries null buffers, so it cannot touch memory whatever
    order the checks run in; host buffers are refused as invalid."""
    fn = noalloc_fn()
    assert fn(None, None, MAX_KEYS + 1, 32, 8, None, None, None) == TOO_LARGE
    assert fn(None, None, 0xFFFFFFFF, 32, 8, None, None, None) == TOO_LARGE
    h = np.zeros(16, np.uint32)
    assert fn(h.ctypes.data, h.ctypes.data, 16, 32, 8, h.ctypes.data, h.ctypes.data, None) == 1
