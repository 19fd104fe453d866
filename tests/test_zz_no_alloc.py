"""The allocation-free extz2 entry point against the allocating one.

hg_ksw_extz2_noalloc serves callers that cannot allocate device memory (a
framework pool allocator that must see every allocation, or a latency-bound
loop that cannot take cudaFree's device-wide synchronisation).  Its scratch
is one fixed array per GPU that every call reuses, so this test makes two
calls in a row - a larger alignment, then a smaller one that would expose
any state left behind by the first - and checks both, through the C ABI,
against hg_ksw_extz2 (bit-exact: the path is integer).  Both entry points run
the same warp kernel, so the reference's own golden extz2 vectors are checked
too, on a non-default stream, and so are the CIGAR-capacity marker and the
refusal of codes >= m.  It is collected last so that a failure here does not
stop the rest of the suite."""
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


def _run(fn, torch, q, t, w, zdrop, eb, flag, cap, stream=None, guard=0):
    dm = torch.from_numpy(MAT.copy()).cuda()
    dq = torch.from_numpy(np.ascontiguousarray(q, np.uint8)).cuda()
    dt = torch.from_numpy(np.ascontiguousarray(t, np.uint8)).cuda()
    dez = torch.full((11,), -7, dtype=torch.int32, device="cuda")
    dcig = torch.full((cap + guard,), -5, dtype=torch.int32, device="cuda")
    err = C.create_string_buffer(256)
    torch.cuda.synchronize()
    rc = fn(len(q), dq.data_ptr(), len(t), dt.data_ptr(), 5, dm.data_ptr(), 6, 2, w, zdrop, eb, flag,
            dez.data_ptr(), dcig.data_ptr(), cap, stream, err, 256)
    assert rc == 0, err.value.decode()
    torch.cuda.synchronize()
    return dez.cpu().numpy(), dcig.cpu().numpy().view(np.uint32)


def test_noalloc_golden_vectors_on_a_side_stream(gpu, golden):
    """The reference's own extz2 outputs (random flags, bands, z-drop, end
    bonus), enqueued on a torch-created non-default stream."""
    torch = pytest.importorskip("torch")
    fn = _entry(gpu.lib())
    g = golden.load("ksw_extz2.npz")
    side = torch.cuda.Stream()
    checked = 0
    for i in range(0, len(g["params"]), 7):
        q = g["q"][g["q_off"][i]:g["q_off"][i + 1]]
        t = g["t"][g["t_off"][i]:g["t_off"][i + 1]]
        w, zdrop, eb, flag = (int(x) for x in g["params"][i])
        if not flag & 0x04:
            continue
        want = g["cigar"][g["cigar_off"][i]:g["cigar_off"][i + 1]]
        cap = len(q) + len(t) + 4
        with torch.cuda.stream(side):
            ez, cig = _run(fn, torch, q, t, w, zdrop, eb, flag, cap, stream=side.cuda_stream)
        assert np.array_equal(ez[:10], g["ez"][i]), i
        assert ez[10] == len(want), i
        assert np.array_equal(cig[:len(want)], want), i
        checked += 1
    assert checked >= 50


def test_noalloc_cigar_capacity_marker(gpu):
    """A CIGAR longer than cap reports a length above cap and writes nothing
    past the first cap words."""
    torch = pytest.importorskip("torch")
    fn = _entry(gpu.lib())
    rng = np.random.default_rng(7)
    q = rng.integers(0, 4, 300).astype(np.uint8)  # unrelated sequences: a long CIGAR
    t = rng.integers(0, 4, 280).astype(np.uint8)
    _, full = gpu.ksw_extz2(q, t, 5, MAT, 6, 2, -1, -1, 0, 0x06)
    assert len(full) > 6
    cap = 4
    ez, cig = _run(fn, torch, q, t, -1, -1, 0, 0x06, cap, guard=64)
    assert ez[10] > cap
    assert np.all(cig[cap:] == np.uint32(0xFFFFFFFB))  # the -5 fill is untouched


def test_noalloc_refuses_codes_of_m_or_more(gpu):
    """Codes >= m would index past the m x m matrix: the kernel checks them,
    computes nothing and reports -1 as the CIGAR length."""
    torch = pytest.importorskip("torch")
    fn = _entry(gpu.lib())
    q = np.array([0, 1, 2, 3, 7, 1], np.uint8)
    t = np.array([0, 1, 2, 3, 1], np.uint8)
    ez, cig = _run(fn, torch, q, t, -1, -1, 0, 0x06, 16)
    assert ez[10] == -1
    assert np.all(cig == np.uint32(0xFFFFFFFB))
    # the scratch is still usable by the next call
    q2, t2 = _case(np.random.default_rng(3), 90, 95, 0.0)
    ez_ref, cig_ref = gpu.ksw_extz2(q2, t2, 5, MAT, 6, 2, -1, -1, 0, 0x06)
    ez2, cig2 = _run(fn, torch, q2, t2, -1, -1, 0, 0x06, 200)
    assert np.array_equal(ez2[:10], ez_ref) and np.array_equal(cig2[:ez2[10]], cig_ref)
