"""The allocation-free entry point, mcfl_batch_run_noalloc.

Callers that cannot allocate device memory (inside another framework's
memory pool, or handed only device buffers) use this variant of the batched
excitation run: its scratch is a static device array inside the library, and
the caller provides inputs and outputs on the device.  Here the device
buffers come from torch, and the results must equal those of the allocating
entry point (mcfl_batch_run, same math, same kernel variant) bit for bit —
the tolerance of every other parity test of the exact kernel, and the
fast-math kernel is as deterministic — on two calls in a row, since the
calls share and reuse the static scratch.  The second call must leave the
device's free memory and torch's allocated memory unchanged.  Invalid
arguments are rejected before anything touches the GPU.  This file is
collected last so that a run stopping at its first failure has run every
other test before it.
"""
import ctypes

import numpy as np
import pytest

import cudamcfl_gb300 as mc
from tests import cases


def _runs(case):
    dx, dy, nx, ny, x0, y0 = case.det
    det = mc.Detector(x0, y0, dx, dy, nx, ny)
    srcs = [(-0.3, 0.1), (0.0, 0.0), (0.25, -0.2), (0.5, 0.5)]
    budgets = [4000, 15000, 7000, 900]
    return [mc.run_desc(b, source=(x, y, 0.0), det=det, seed_exc=300 + i, start_weight=case.start_weight())
            for i, ((x, y), b) in enumerate(zip(srcs, budgets))]


def _ptr(t):
    return ctypes.c_void_p(t if isinstance(t, int) else t.data_ptr())


def _noalloc(lib, case, runs, labels, prop, R, T, st, stream, math=mc.MATH_EXACT):
    nx, ny, nz = case.dims
    e = np.float32(case.esp)
    vox = (ctypes.c_float * 3)(*([float(case.grid)] * 3))
    arr = (mc.RunDesc * len(runs))(*runs)
    return lib.mcfl_batch_run_noalloc(
        math, _ptr(labels), _ptr(prop), nx, ny, nz,
        ctypes.c_float(float(np.float32(2) * e)), ctypes.c_float(float(np.float32(2) * e)), ctypes.c_float(float(e)),
        vox, len(case.bulks()) - 2, arr, len(runs), _ptr(R), _ptr(T), _ptr(st), ctypes.c_void_p(stream))


def _bind(lib):
    lib.mcfl_batch_run_noalloc.restype = ctypes.c_int
    lib.mcfl_batch_run_noalloc.argtypes = [
        ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_float,
        ctypes.c_float, ctypes.c_float, ctypes.POINTER(ctypes.c_float), ctypes.c_int, ctypes.POINTER(mc.RunDesc),
        ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]


@pytest.mark.gpu
@pytest.mark.parametrize("math", [mc.MATH_EXACT, mc.MATH_FAST])
def test_noalloc_equals_batch_run_on_two_calls(math):
    torch = pytest.importorskip("torch")
    from cudamcfl_gb300 import build
    build.build()
    lib = mc.load()
    _bind(lib)
    case = cases.sphere()
    runs = _runs(case)
    ctx = mc.Context(math=math)
    ctx.set_option("variant", 0)  # the kernel variant the allocation-free call launches
    med = case.engine_medium(ctx)
    ref, _ = mc.batch_run(ctx, med, runs, mc.SCHEDULE_BATCHED)
    med.free()
    ctx.close()

    dev = torch.device("cuda", 0)
    labels = torch.from_numpy(np.ascontiguousarray(case.labels).ravel()).to(dev)
    prop = torch.tensor([[b.mutr, b.mua, b.g, b.n] for b in case.bulks()], dtype=torch.float32, device=dev)
    xy = case.det[2] + case.det[2] * case.det[3]
    n = len(runs)
    R = torch.full((n * xy,), -1, dtype=torch.int64, device=dev)  # garbage: the call must clear it
    T = torch.full((n * xy,), -1, dtype=torch.int64, device=dev)
    st = torch.full((n * mc.NSTATS,), -1, dtype=torch.int64, device=dev)
    stream = torch.cuda.current_stream(dev).cuda_stream
    for call in range(2):
        torch.cuda.synchronize(dev)
        free0, _ = torch.cuda.mem_get_info(dev)
        alloc0 = torch.cuda.memory_allocated(dev)
        assert _noalloc(lib, case, runs, labels, prop, R, T, st, stream, math) == mc.OK, mc.last_error()
        torch.cuda.synchronize(dev)
        if call == 1:  # the first call of the process may load kernels; the second allocates nothing
            assert torch.cuda.mem_get_info(dev)[0] == free0
            assert torch.cuda.memory_allocated(dev) == alloc0
        Rh = R.cpu().numpy().view(np.uint64).reshape(n, xy)
        Th = T.cpu().numpy().view(np.uint64).reshape(n, xy)
        Sh = st.cpu().numpy().view(np.uint64).reshape(n, mc.NSTATS)
        for i in range(n):
            assert np.array_equal(Rh[i], ref[i]["Rd"]), (call, i)
            assert np.array_equal(Th[i], ref[i]["Tt"]), (call, i)
            assert Sh[i][0] == runs[i].photons
            assert tuple(int(v) for v in Sh[i]) == tuple(ref[i]["stats"][k] for k in mc.STAT_NAMES)


@pytest.mark.gpu
def test_noalloc_rejects_more_than_max_jobs():
    torch = pytest.importorskip("torch")
    lib = mc.load()
    _bind(lib)
    case = cases.tiny()
    runs = _runs(case) * 17  # 68 > 64
    dev = torch.device("cuda", 0)
    labels = torch.zeros(case.labels.size, dtype=torch.uint8, device=dev)
    prop = torch.zeros((4, 4), dtype=torch.float32, device=dev)
    buf = torch.zeros(8, dtype=torch.int64, device=dev)
    rc = _noalloc(lib, case, runs, labels, prop, buf, buf, buf, torch.cuda.current_stream(dev).cuda_stream)
    assert rc == mc.E_RANGE
    assert "MCFL_NOALLOC_MAX_JOBS" in mc.last_error()


def test_noalloc_rejects_bad_arguments_before_any_gpu_work():
    """Misaligned buffers and a bad detector on any run are refused by the
    host checks, before the call touches the GPU (the addresses below are
    never dereferenced)."""
    from cudamcfl_gb300 import build
    build.build()
    lib = mc.load()
    _bind(lib)
    case = cases.tiny()
    runs = _runs(case)
    good = dict(labels=0x10000, prop=0x20000, R=0x30000, T=0x40000, st=0x50000)

    def call(**kw):
        a = dict(good, **kw)
        return _noalloc(lib, case, kw.pop("runs", runs), a["labels"], a["prop"], a["R"], a["T"], a["st"], 0)

    assert call(prop=0x20004) == mc.E_ARG and "16-byte" in mc.last_error()
    assert call(R=0x30004) == mc.E_ARG and "8-byte" in mc.last_error()
    assert call(st=0x50002) == mc.E_ARG
    bad = _runs(case)
    bad[2].det.dx = 0.0
    assert call(runs=bad) == mc.E_ARG and "detector" in mc.last_error()
