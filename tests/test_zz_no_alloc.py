"""The allocation-free extz2 entry point against the allocating one.

hg_ksw_extz2_noalloc serves callers that cannot allocate device memory (a
framework pool allocator that must see every allocation, or a latency-bound
loop that cannot take cudaFree's device-wide synchronisation).  Its scratch
is one fixed array per GPU that every call reuses, so this test makes two
calls in a row - a larger alignment, then a smaller one that would expose
any state left behind by the first - and checks both, through the C ABI,
against hg_ksw_extz2 (bit-exact: the path is integer).  It is collected last
so that a failure here does not stop the rest of the suite."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

MAT = np.array([5, -4, -4, -4, 0, -4, 5, -4, -4, 0, -4, -4, 5, -4, 0, -4, -4, -4, 5, 0, 0, 0, 0, 0, 0], np.int8)


def _entry(lib):
    fn = lib.hg_ksw_extz2_noalloc
    vp, i32 = C.c_void_p, C.c_int
    fn.argtypes = [i32, vp, i32, vp, C.c_int8, vp, C.c_int8, C.c_int8, i32, i32, i32, i32, vp, vp, C.c_int64, vp,
                   C.c_char_p, C.c_int64]
    fn.restype = i32
    return fn


def _case(rng, qn, tn, n_rate):
    q = rng.integers(0, 4, qn).astype(np.uint8)
    t = np.resize(q, tn).copy()
    m = rng.random(tn) < 0.08
    t[m] = rng.integers(0, 5, int(m.sum()))
    t[rng.random(tn) < n_rate] = 4
    return q, t


def test_noalloc_matches_allocating_entry_point_twice(gpu):
    torch = pytest.importorskip("torch")
    fn = _entry(gpu.lib())
    rng = np.random.default_rng(2024)
    cases = [(*_case(rng, 420, 390, 0.01), 60, 0x06), (*_case(rng, 75, 81, 0.0), -1, 0x04)]
    dm = torch.from_numpy(MAT.copy()).cuda()
    for q, t, w, flag in cases:
        ez_ref, cig_ref = gpu.ksw_extz2(q, t, 5, MAT, 6, 2, w, -1, 0, flag)
        cap = len(q) + len(t) + 4
        dq = torch.from_numpy(q).cuda()
        dt = torch.from_numpy(t).cuda()
        dez = torch.full((11,), -7, dtype=torch.int32, device="cuda")
        dcig = torch.zeros(cap, dtype=torch.int32, device="cuda")
        err = C.create_string_buffer(256)
        torch.cuda.synchronize()
        rc = fn(len(q), dq.data_ptr(), len(t), dt.data_ptr(), 5, dm.data_ptr(), 6, 2, w, -1, 0, flag,
                dez.data_ptr(), dcig.data_ptr(), cap, None, err, 256)
        assert rc == 0, err.value.decode()
        torch.cuda.synchronize()
        ez = dez.cpu().numpy()
        n = int(ez[10])
        assert 0 < n <= cap
        cig = dcig.cpu().numpy()[:n].view(np.uint32)
        assert np.array_equal(ez[:10], ez_ref)
        assert np.array_equal(cig, cig_ref)


def test_noalloc_rejects_scratch_above_limit(gpu):
    fn = _entry(gpu.lib())
    err = C.create_string_buffer(256)
    # a 3000 x 3000 full-band alignment needs far more than the static scratch;
    # it is refused on the host before any device pointer is touched
    rc = fn(3000, 1, 3000, 1, 5, 1, 6, 2, -1, -1, 0, 0x06, 1, 1, 6004, None, err, 256)
    assert rc == 4
    assert b"static limit" in err.value
