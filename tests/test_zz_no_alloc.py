"""The allocation-free radix sort (vcr_radix_sort_pairs_noalloc).

It exists for callers that may not allocate device memory themselves or let
a library do it (a host application that owns all device memory through its
own pool, a render loop that must not allocate after start-up, a plug-in
handed buffers but no allocator).  Its working memory is a fixed device
array inside the library, so it is limited to VCR_SORT_NOALLOC_MAX_KEYS
pairs per call and calls must not overlap on the GPU.

These tests call it through the C-ABI and check that its output equals the
context-based vcr_radix_sort_pairs bit for bit (integer work: tolerance 0),
on two calls in a row with different inputs, so the second call cannot
depend on what the first left in the shared array.  A caller without a
context learns of a device-side wait that ran out from
vcr_sort_noalloc_status, which the tests check on every call, and make
happen once on purpose.  This file is collected last on purpose.
"""
import ctypes as C

import numpy as np
import pytest

import vcr
from vcr import _abi

pytestmark = pytest.mark.gpu

MAX_KEYS = 1 << 20  # VCR_SORT_NOALLOC_MAX_KEYS in include/vcr/abi.h


def _noalloc(dk, dv, ko, vo, n, begin=0, end=32, stream=0):
    return vcr.lib().vcr_radix_sort_pairs_noalloc(
        C.c_void_p(dk), C.c_void_p(dv) if dv else None, C.c_void_p(ko), C.c_void_p(vo), n, begin, end,
        C.c_void_p(stream))


def _status(stream=0):
    return vcr.lib().vcr_sort_noalloc_status(C.c_void_p(stream))


def _case(torch, cuda, n, seed, with_vals, bits):
    g = torch.Generator(device=cuda).manual_seed(seed)
    keys = torch.randint(-(1 << 31), (1 << 31) - 1, (max(n, 1),), dtype=torch.int32, device=cuda, generator=g)
    vals = torch.randint(-(1 << 31), (1 << 31) - 1, (max(n, 1),), dtype=torch.int32, device=cuda, generator=g)
    return keys, (vals if with_vals else None), bits


def test_noalloc_sort_matches_context_sort_twice(cuda):
    import torch

    cases = [(MAX_KEYS, 11, True, (0, 32)), (123457, 12, False, (0, 30))]
    with vcr.Context() as ctx:
        for n, seed, with_vals, bits in cases:
            keys, vals, (b0, b1) = _case(torch, cuda, n, seed, with_vals, bits)
            ref_k = torch.empty_like(keys)
            ref_v = torch.empty_like(keys)
            ctx.radix_sort_pairs(keys.data_ptr(), vals.data_ptr() if vals is not None else None, ref_k.data_ptr(),
                                 ref_v.data_ptr(), n, b0, b1)
            ctx.synchronize()
            out_k = torch.full_like(keys, 7)
            out_v = torch.full_like(keys, 7)
            st = _noalloc(keys.data_ptr(), vals.data_ptr() if vals is not None else 0, out_k.data_ptr(),
                          out_v.data_ptr(), n, b0, b1)
            assert st == _abi.OK, vcr.lib().vcr_last_error(None)
            assert _status() == _abi.OK, vcr.lib().vcr_last_error(None)
            torch.cuda.synchronize()
            assert torch.equal(out_k[:n], ref_k[:n])
            assert torch.equal(out_v[:n], ref_v[:n])
            if vals is None:  # the payload is the stable permutation of the keys' bits [b0, b1)
                k = keys[:n].cpu().numpy().view(np.uint32)
                perm = np.argsort(k & np.uint32((1 << b1) - 1), kind="stable").astype(np.uint32)
                np.testing.assert_array_equal(out_v[:n].cpu().numpy().view(np.uint32), perm)


@pytest.mark.parametrize("end_bit", [28, 24])
def test_noalloc_sort_in_place_and_on_a_stream(cuda, end_bit):
    """In place with an even (4) and an odd (3) pass count: the order is the
    stable argsort of the keys' bits [0, end_bit)."""
    import torch

    n = 300001
    keys, _, _ = _case(torch, cuda, n, 21, False, (0, 32))
    k0 = keys.cpu().numpy().view(np.uint32).copy()
    vals = torch.arange(n, dtype=torch.int32, device=cuda)
    s = torch.cuda.Stream()
    s.wait_stream(torch.cuda.current_stream())  # the inputs were written on the default stream
    with torch.cuda.stream(s):
        st = _noalloc(keys.data_ptr(), vals.data_ptr(), keys.data_ptr(), vals.data_ptr(), n, 0, end_bit,
                      stream=s.cuda_stream)
        assert st == _abi.OK, vcr.lib().vcr_last_error(None)
        assert _status(s.cuda_stream) == _abi.OK
    s.synchronize()
    perm = np.argsort(k0 & np.uint32((1 << end_bit) - 1), kind="stable").astype(np.uint32)
    np.testing.assert_array_equal(vals.cpu().numpy().view(np.uint32), perm)
    np.testing.assert_array_equal(keys.cpu().numpy().view(np.uint32), k0[perm])


def test_noalloc_sort_rejects_sizes_beyond_its_scratch(cuda):
    import torch

    d = torch.zeros(4, dtype=torch.int32, device=cuda)
    st = _noalloc(d.data_ptr(), 0, d.data_ptr(), d.data_ptr(), MAX_KEYS + 1)
    assert st == _abi.ERR_CAPACITY
    assert b"exceed the fixed scratch" in vcr.lib().vcr_last_error(None)
    assert _noalloc(d.data_ptr(), 0, d.data_ptr(), d.data_ptr(), 0) == _abi.OK


def test_noalloc_sort_reports_a_wait_that_ran_out(cuda):
    """With the look-back limit at zero polls a tile gives up on a
    predecessor that has not published yet: the sort's order is then
    unspecified (it stays inside its buffers) and vcr_sort_noalloc_status
    says so.  With the default limit restored, the next sort is exact."""
    import torch

    n = MAX_KEYS
    keys, _, _ = _case(torch, cuda, n, 31, False, (0, 32))
    out_k = torch.empty_like(keys)
    out_v = torch.empty_like(keys)
    try:
        vcr.set_wait_limits(sort_lookback=0)
        seen = []
        for _ in range(3):
            assert _noalloc(keys.data_ptr(), 0, out_k.data_ptr(), out_v.data_ptr(), n) == _abi.OK
            seen.append(_status())
            if seen[-1] == _abi.ERR_TIMEOUT:
                break
        assert _abi.ERR_TIMEOUT in seen, seen
        assert b"look-back wait ran out" in vcr.lib().vcr_last_error(None)
        assert _status() == _abi.OK  # the word was cleared
    finally:
        vcr.set_wait_limits()
    assert _noalloc(keys.data_ptr(), 0, out_k.data_ptr(), out_v.data_ptr(), n) == _abi.OK
    assert _status() == _abi.OK
    k = keys.cpu().numpy().view(np.uint32)
    perm = np.argsort(k, kind="stable").astype(np.uint32)
    np.testing.assert_array_equal(out_v.cpu().numpy().view(np.uint32), perm)
