"""colo_table_pi_static, the allocation-free participation-index entry point,
against colo_mine's own numerators and PI (colo_result_level) on the
instance tables colo_mine kept (colo_result_table).

The entry point keeps its bitmaps in one fixed device array shared by all
calls, so the checks run many calls back to back, big tables before small
ones and the same table twice, to show that every call starts from cleared
scratch.  Device buffers come from torch: the test may allocate, the entry
point does not.
"""
import ctypes as C

import numpy as np
import pytest

import colo
from colo import gen

CAPACITY_WORDS = 1 << 20   # COLO_TABLE_PI_STATIC_WORDS


def _features(fid):
    fid = np.asarray(fid)
    starts = np.concatenate([[0], np.flatnonzero(np.diff(fid) != 0) + 1]).astype(np.uint32)
    counts = np.diff(np.concatenate([starts, [len(fid)]])).astype(np.uint32)
    return starts, counts


class _Caller:
    """Calls the entry point through the C ABI with torch-owned device buffers."""

    def __init__(self, torch):
        self.torch = torch
        self.lib = colo.load()
        self.num = torch.empty(32, dtype=torch.int64, device="cuda")
        self.pi = torch.empty(1, dtype=torch.float32, device="cuda")

    def __call__(self, table, cand, starts, counts):
        torch = self.torch
        k = len(cand)
        t = torch.from_numpy(np.ascontiguousarray(table, dtype=np.uint32).view(np.int32)).cuda()
        fs = np.ascontiguousarray(starts[cand], dtype=np.uint32)
        fc = np.ascontiguousarray(counts[cand], dtype=np.uint32)
        self.num.fill_(-7)
        self.pi.fill_(-7.0)
        stream = torch.cuda.current_stream().cuda_stream
        st = self.lib.colo_table_pi_static(t.data_ptr() if t.numel() else None, table.shape[0], k,
                                           fs.ctypes.data_as(C.POINTER(C.c_uint32)),
                                           fc.ctypes.data_as(C.POINTER(C.c_uint32)),
                                           self.num.data_ptr(), self.pi.data_ptr(), stream)
        assert st == 0, colo.STATUS.get(st, st)
        torch.cuda.synchronize()
        num = self.num[:k].cpu().numpy().view(np.uint64).copy()
        pi = self.pi.cpu().numpy().copy()
        return num, pi[0]


def _mined(ctx, wl):
    ds = colo.Dataset.from_arrays(ctx, wl.x, wl.y, wl.fid, wl.bounds)
    res = ctx.mine(ds, colo.default_params(wl.R, wl.thr, colo.MODE_BATCHED, max_size=wl.max_size,
                                           keep_tables=True))
    starts, counts = _features(wl.fid)
    assert len(starts) == ctx.lib.colo_dataset_num_features(ds.h)
    cases = []
    for lev in res.levels:
        for c, t in lev.tables.items():
            cases.append((t, lev.cand[c].astype(np.int64), lev.num[c], lev.pi[c]))
    return cases, starts, counts


@pytest.mark.gpu
@pytest.mark.parametrize("cfg,scale", [(0, 1.0), (1, 0.02)])
def test_static_entry_matches_mining_numerators(cfg, scale):
    torch = pytest.importorskip("torch")
    ctx = colo.Context(0)
    cases, starts, counts = _mined(ctx, gen.config(cfg, scale=scale))
    assert cases, "no instance tables kept"
    call = _Caller(torch)
    # largest table first, so later small calls run on scratch full of old bits
    order = sorted(range(len(cases)), key=lambda i: -cases[i][0].shape[0])
    seen_k = set()
    for i in order:
        table, cand, num, pi = cases[i]
        got_num, got_pi = call(table, cand, starts, counts)
        assert np.array_equal(got_num, num), (cand, got_num, num)
        assert np.float32(got_pi).view(np.uint32) == np.float32(pi).view(np.uint32), (cand, got_pi, pi)
        seen_k.add(len(cand))
    # two calls in a row on the same table after a different one: same answer
    big, small = cases[order[0]], cases[order[-1]]
    for table, cand, num, pi in (big, small, small, big, big):
        got_num, got_pi = call(table, cand, starts, counts)
        assert np.array_equal(got_num, num)
        assert np.float32(got_pi).view(np.uint32) == np.float32(pi).view(np.uint32)
    assert 2 in seen_k


@pytest.mark.gpu
def test_static_entry_takes_no_device_memory():
    """The device's free memory does not drop across calls of the entry point.

    Everything the calls touch is in place first: the torch buffers, and the
    library's module with its scratch array (loaded by a warm-up call).  A
    cudaMalloc on the call path would show as less free memory afterwards;
    other tests' contexts freed meanwhile can only raise it.
    """
    import gc

    torch = pytest.importorskip("torch")
    ctx = colo.Context(0)
    cases, starts, counts = _mined(ctx, gen.config(0))
    call = _Caller(torch)
    dev_tables = [(torch.from_numpy(np.ascontiguousarray(t, np.uint32).view(np.int32)).cuda(), t.shape[0],
                   np.ascontiguousarray(starts[c], np.uint32), np.ascontiguousarray(counts[c], np.uint32), num)
                  for t, c, num, _ in cases]
    lib = call.lib
    stream = torch.cuda.current_stream().cuda_stream

    def run_all():
        for t, rows, fs, fc, _ in dev_tables:
            st = lib.colo_table_pi_static(t.data_ptr(), rows, len(fs), fs.ctypes.data_as(C.POINTER(C.c_uint32)),
                                          fc.ctypes.data_as(C.POINTER(C.c_uint32)), call.num.data_ptr(),
                                          call.pi.data_ptr(), stream)
            assert st == 0, colo.STATUS.get(st, st)
        torch.cuda.synchronize()

    run_all()                      # warm-up: module load, scratch address lookup
    gc.collect()
    gc.disable()
    try:
        free0, _ = torch.cuda.mem_get_info()
        for _ in range(3):
            run_all()
        free1, _ = torch.cuda.mem_get_info()
    finally:
        gc.enable()
    assert free1 >= free0, (free0, free1)
    t, rows, fs, fc, num = dev_tables[-1]
    assert np.array_equal(call.num[:len(fs)].cpu().numpy().view(np.uint64), num)


@pytest.mark.gpu
def test_static_entry_flags_ids_outside_members():
    torch = pytest.importorskip("torch")
    call = _Caller(torch)
    starts = np.array([0, 100, 250], np.uint32)
    counts = np.array([100, 150, 50], np.uint32)
    good = np.array([[0, 100, 250], [5, 120, 251], [99, 249, 299]], np.uint32)
    num, pi = call(good, np.array([0, 1, 2]), starts, counts)
    # num0 = A0 = |{0, 5}| (bit n-1 = 99 is outside the window); num_j = last_{j-1} + A_j
    assert num.tolist() == [2, 1 + 2, 1 + 2]
    bad = good.copy()
    bad[1, 1] = 300   # not an instance of member 1
    num, pi = call(bad, np.array([0, 1, 2]), starts, counts)
    assert (num == np.iinfo(np.uint64).max).all() and np.isnan(pi)
    num, pi = call(good, np.array([0, 1, 2]), starts, counts)   # the next call is clean again
    assert num.tolist() == [2, 3, 3]


def test_static_entry_rejects_sizes_beyond_its_array():
    lib = colo.load()
    k = 2
    fs = np.zeros(k, np.uint32)
    fc = np.array([CAPACITY_WORDS * 32 - 31, 64], np.uint32)   # ceil/32 sums to the maximum + 2
    dummy = C.c_void_p(16)   # never dereferenced: the size check comes first
    st = lib.colo_table_pi_static(dummy, 1, k, fs.ctypes.data_as(C.POINTER(C.c_uint32)),
                                  fc.ctypes.data_as(C.POINTER(C.c_uint32)), dummy, dummy, None)
    assert st == 8   # COLO_ERR_CAPACITY
    st = lib.colo_table_pi_static(dummy, 1, 1, fs.ctypes.data_as(C.POINTER(C.c_uint32)),
                                  fc.ctypes.data_as(C.POINTER(C.c_uint32)), dummy, dummy, None)
    assert st == 1   # k = 1: COLO_ERR_ARG
