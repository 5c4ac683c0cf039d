"""sgba_total_cost_noalloc: the allocation-free total cost against the
oracle's calc_total_cost (the FP64 CPU restatement of the reference,
crates/sophus_opt/src/nlls/cost/cost_fn.rs:403-433) and against the cost
that sgba_get_cost reports for the same variables.

The file name sorts last so that the GPU test also runs after every other
test has used the device; it passes alone in a fresh process as well.
"""
import ctypes as C

import numpy as np
import pytest

from conftest import fixed_iter_params

MAX_CAMS = 4096       # the static scratch's camera capacity, stated in sgba.h
RTOL = 1e-10          # both sides are float-float sums of the same terms, summed in other orders


def _bind(pkg):
    f = pkg.native.lib().sgba_total_cost_noalloc
    f.argtypes = [C.c_int32, C.c_void_p, C.c_int32, C.c_void_p, C.c_int64, C.c_void_p, C.c_void_p,
                  C.c_void_p, C.POINTER(C.c_double), C.c_double, C.c_void_p, C.c_void_p]
    f.restype = C.c_int32
    return f


def test_rejects_more_cameras_than_the_scratch_holds(pkg):
    """Checked on the host before any CUDA call (runs without a GPU)."""
    f = _bind(pkg)
    intr = (C.c_double * 4)(500.0, 500.0, 320.0, 240.0)
    st = f(MAX_CAMS + 1, None, 0, None, 0, None, None, None, intr, 1.0, None, None)
    assert st == pkg.native.ERR_INVALID_ARGUMENT
    assert "4096" in pkg.native.last_error()
    st = f(2, None, 0, None, 0, None, None, None, intr, 1.0, None, None)
    assert st == pkg.native.ERR_INVALID_ARGUMENT and "NULL" in pkg.native.last_error()


def test_rejects_misaligned_pointers_and_unrepresentable_huber(pkg):
    """Also host-side checks, before any CUDA call: the kernels load obs_uv as
    16-byte pairs, and compare with the Huber threshold in float."""
    f = _bind(pkg)
    intr = (C.c_double * 4)(500.0, 500.0, 320.0, 240.0)
    base = 1 << 20  # never dereferenced: the checks reject first
    args = dict(poses=base, points=base + 256, cam=base + 512, pt=base + 768, uv=base + 1024, out=base + 1280)

    def call(huber=1.0, **kw):
        a = dict(args, **kw)
        return f(2, a["poses"], 1, a["points"], 1, a["cam"], a["pt"], a["uv"], intr, huber, a["out"], None)

    assert call(uv=base + 1024 + 8) == pkg.native.ERR_INVALID_ARGUMENT  # 8 but not 16 bytes
    assert "misaligned" in pkg.native.last_error()
    assert call(poses=base + 4) == pkg.native.ERR_INVALID_ARGUMENT
    assert call(cam=base + 514) == pkg.native.ERR_INVALID_ARGUMENT
    assert call(huber=1e-40) == pkg.native.ERR_INVALID_ARGUMENT  # positive, below the normal floats
    assert "huber" in pkg.native.last_error()


def _expected_cost(pkg, prob):
    with pkg.native.Problem(prob, device=0) as gp:
        gp.init(fixed_iter_params(pkg, 1, prob.initial_lm_damping))
        return gp.cost()


def _device_arrays(torch, prob):
    dev = torch.device("cuda", 0)
    t = lambda a, dt: torch.from_numpy(np.ascontiguousarray(a, dtype=dt)).to(dev)  # noqa: E731
    return dict(poses=t(prob.poses, np.float64), points=t(prob.points, np.float64),
                cam=t(prob.obs_cam, np.int32), pt=t(prob.obs_pt, np.int32), uv=t(prob.obs_uv, np.float64),
                out=torch.full((1,), float("nan"), dtype=torch.float64, device=dev))


def _call(pkg, f, torch, prob, a):
    intr = (C.c_double * 4)(*[float(v) for v in prob.intrinsics])
    huber = float(prob.huber_delta) if prob.huber_delta is not None else 0.0
    stream = torch.cuda.current_stream(0).cuda_stream
    st = f(prob.n_cam, a["poses"].data_ptr(), prob.n_pt, a["points"].data_ptr(), prob.n_obs,
           a["cam"].data_ptr(), a["pt"].data_ptr(), a["uv"].data_ptr(), intr, huber, a["out"].data_ptr(),
           C.c_void_p(stream))
    assert st == pkg.native.OK, pkg.native.last_error()


@pytest.mark.gpu
def test_noalloc_cost_matches_oracle_and_get_cost(pkg, oracle):
    torch = pytest.importorskip("torch")
    torch.cuda.init()
    f = _bind(pkg)
    first = pkg.synth.generate(pkg.synth.CIRCLE, seed=pkg.synth.BASE_SEED + 11)
    second = pkg.synth.generate(pkg.synth.LOOP, n_cam=300, n_pt=3000, seed=pkg.synth.BASE_SEED + 12)
    second.huber_delta = 0.0  # no robust kernel on the second problem
    probs = (first, second)
    expected = [_expected_cost(pkg, p) for p in probs]
    ora = [oracle.total_cost(p) for p in probs]  # f64 calc_total_cost, Huber and no kernel
    arrays = [_device_arrays(torch, p) for p in probs]
    # two calls in a row on one stream, different sizes, then read both
    _call(pkg, f, torch, first, arrays[0])
    _call(pkg, f, torch, second, arrays[1])
    torch.cuda.synchronize()
    got = [float(a["out"].cpu()[0]) for a in arrays]
    for g, e, o in zip(got, expected, ora):
        assert np.isfinite(g) and abs(g - e) <= RTOL * abs(e), (g, e)
        assert abs(g - o) <= RTOL * abs(o), (g, o)
    # the same inputs again: bit-identical (fixed reduction order)
    _call(pkg, f, torch, first, arrays[0])
    torch.cuda.synchronize()
    assert float(arrays[0]["out"].cpu()[0]) == got[0]


@pytest.mark.gpu
def test_noalloc_out_of_range_index_gives_nan(pkg):
    """The kernel checks every index and never dereferences a bad one."""
    torch = pytest.importorskip("torch")
    f = _bind(pkg)
    prob = pkg.synth.generate(pkg.synth.CIRCLE, seed=pkg.synth.BASE_SEED + 13)
    prob.obs_cam = prob.obs_cam.copy()
    prob.obs_cam[17] = prob.n_cam  # one past the last camera
    a = _device_arrays(torch, prob)
    _call(pkg, f, torch, prob, a)
    torch.cuda.synchronize()
    assert np.isnan(float(a["out"].cpu()[0]))
