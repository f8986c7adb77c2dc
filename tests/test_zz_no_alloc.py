"""nsg_sort_device_noalloc, the allocation-free sort of caller-owned device columns,
against the context sort nsg_sort_particles and the oracle on the same inputs, and
with the device's free memory and torch's allocation counters unchanged by a call.
The file name makes it collect last, so that it runs both alone and after every
other test."""
import ctypes as C

import numpy as np
import pytest

MAX_N = 1 << 20


def _inputs(n, seed):
    rng = np.random.default_rng(seed)
    r = rng.random(n) * 10.0
    vr = rng.standard_normal(n)
    ell = rng.random(n)
    aux = rng.standard_normal(n)
    if n >= 64:
        r[rng.choice(n, n // 8, replace=False)] = 0.25      # ties broken by id
        r[:8:2] = -0.0                                       # -0.0 and +0.0 are one key
        r[1:8:2] = 0.0
        r[8] = np.inf
        r[9] = np.nan                                        # NaN sorts last
    ids = rng.permutation(n).astype(np.int32)
    return r, vr, ell, ids, aux


def _context_sort(nsg, r, vr, ell, ids, aux):
    rows = [r, vr, ell, ids.astype(np.float64)] + ([aux] if aux is not None else [])
    table = np.ascontiguousarray(np.stack(rows))
    with nsg.Context(nsg.default_params(carry_aux=int(aux is not None))) as c:
        nsg.sort_particles(c, table)
    out = [table[0], table[1], table[2], table[3].astype(np.int32)]
    return out + ([table[4]] if aux is not None else [])


def _device(torch, cols):
    return [torch.from_numpy(np.ascontiguousarray(x)).cuda() for x in cols]


def _call(nsg, dev, n, stream):
    ptr = [C.c_void_p(t.data_ptr()) for t in dev]
    aux = ptr[4] if len(ptr) > 4 else None
    return nsg.lib().nsg_sort_device_noalloc(ptr[0], ptr[1], ptr[2], ptr[3], aux, n, C.c_void_p(stream))


def _same(a, b):
    a, b = np.asarray(a), np.asarray(b)
    return a.dtype == b.dtype and a.shape == b.shape and np.array_equal(a.view(np.uint8), b.view(np.uint8))


def test_rejects_bad_sizes_without_device_work(nsg):
    L = nsg.lib()
    assert L.nsg_sort_device_noalloc(None, None, None, None, None, MAX_N + 1, None) == nsg.NSG_EINVAL
    assert b"1048576" in L.nsg_last_error(None)
    assert L.nsg_sort_device_noalloc(None, None, None, None, None, -1, None) == nsg.NSG_EINVAL
    assert L.nsg_sort_device_noalloc(None, None, None, None, None, 5, None) == nsg.NSG_EINVAL
    assert L.nsg_sort_device_noalloc(None, None, None, None, None, 0, None) == nsg.NSG_OK


@pytest.mark.gpu
def test_two_calls_in_a_row_match_context_sort(nsg, oracle):
    torch = pytest.importorskip("torch")
    a = _inputs(300_001, seed=71)                  # ragged last tile, with aux
    b = _inputs(77_777, seed=72)[:4] + (None,)     # aux NULL
    want_a = _context_sort(nsg, *a)
    want_b = _context_sort(nsg, *b)
    dev_a = _device(torch, a)
    dev_b = _device(torch, b[:4])
    s = torch.cuda.Stream()
    torch.cuda.synchronize()
    assert _call(nsg, dev_a, len(a[0]), s.cuda_stream) == nsg.NSG_OK
    assert _call(nsg, dev_b, len(b[0]), s.cuda_stream) == nsg.NSG_OK
    s.synchronize()
    for got, want in zip(dev_a, want_a):
        assert _same(got.cpu().numpy(), want)
    for got, want in zip(dev_b, want_b):
        assert _same(got.cpu().numpy(), want)
    # and directly against the oracle's (r, id) sort
    for got, want in zip(dev_a, oracle.sort(*a)):
        assert _same(got.cpu().numpy(), want)
    for got, want in zip(dev_b, oracle.sort(*b[:4])):
        assert _same(got.cpu().numpy(), want)


@pytest.mark.gpu
def test_a_call_allocates_no_device_memory(nsg):
    torch = pytest.importorskip("torch")
    cols = _inputs(MAX_N, seed=76)
    dev = _device(torch, cols)
    stream = torch.cuda.current_stream().cuda_stream
    torch.cuda.synchronize()
    assert _call(nsg, dev, MAX_N, stream) == nsg.NSG_OK      # warm: module and scratch loaded
    torch.cuda.synchronize()
    free0 = torch.cuda.mem_get_info()[0]
    allocs0 = torch.cuda.memory_stats().get("allocation.all.allocated", 0)
    assert _call(nsg, dev, MAX_N, stream) == nsg.NSG_OK
    torch.cuda.synchronize()
    assert torch.cuda.mem_get_info()[0] == free0
    assert torch.cuda.memory_stats().get("allocation.all.allocated", 0) == allocs0


@pytest.mark.gpu
def test_largest_size_and_one_past_it(nsg):
    torch = pytest.importorskip("torch")
    cols = _inputs(MAX_N, seed=73)
    want = _context_sort(nsg, *cols)
    dev = _device(torch, cols)
    torch.cuda.synchronize()
    stream = torch.cuda.current_stream().cuda_stream
    assert _call(nsg, dev, MAX_N, stream) == nsg.NSG_OK
    torch.cuda.synchronize()
    for got, w in zip(dev, want):
        assert _same(got.cpu().numpy(), w)
    over = _inputs(MAX_N + 1, seed=74)
    dev = _device(torch, over)
    torch.cuda.synchronize()
    assert _call(nsg, dev, MAX_N + 1, stream) == nsg.NSG_EINVAL
    torch.cuda.synchronize()
    for got, w in zip(dev, over):
        assert _same(got.cpu().numpy(), w)


@pytest.mark.gpu
@pytest.mark.parametrize("n", [1, 2, 31, 2048, 2049])
def test_small_sizes(nsg, n):
    torch = pytest.importorskip("torch")
    cols = _inputs(n, seed=75 + n)
    want = _context_sort(nsg, *cols)
    dev = _device(torch, cols)
    torch.cuda.synchronize()
    assert _call(nsg, dev, n, torch.cuda.current_stream().cuda_stream) == nsg.NSG_OK
    torch.cuda.synchronize()
    for got, w in zip(dev, want):
        assert _same(got.cpu().numpy(), w)
