"""The configurations the benchmark is quoted on, checked against the FP64
oracle at their own sizes (not only on small boxes and round trips):

* 512^3 complex<float> c2c, plain FP32 and the tensor-core (split-BF16) form;
* 512^3 float r2c along dimension 0;
* DCT-II 256^3 float (rtransform<cos>);
* 1024 x 1024 x 512 complex<float> c2c, plain and tensor-core form;
* 512^3 complex<double> c2c.

Inputs as in the benchmark: re / im uniform [-1, 1) for complex data,
standard normal for real data, drawn on the device from fixed seeds.  Each
forward result is compared with the oracle's FP64 transform of the same
input (rel-L2 <= 1e-6 float, <= 1e-12 double, benchmarks/speed3d.h:162-258
conventions: forward unscaled), each backward result (scale::full) with the
input (round trip).  The measured errors are printed in the run summary.
"""
import numpy as np
import pytest

from oracle import heffte_oracle as O

torch = pytest.importorskip("torch")
pytestmark = [pytest.mark.gpu, pytest.mark.slow]

TOL = {0: 1e-6, 1: 1e-12}


def _complex_input(n, prec, seed):
    g = torch.Generator(device="cuda")
    g.manual_seed(seed)
    rdt = torch.float32 if prec == 0 else torch.float64
    re = torch.rand(n, device="cuda", generator=g, dtype=rdt) * 2 - 1
    im = torch.rand(n, device="cuda", generator=g, dtype=rdt) * 2 - 1
    return torch.complex(re, im)


def _real_input(n, seed):
    g = torch.Generator(device="cuda")
    g.manual_seed(seed)
    return torch.randn(n, device="cuda", generator=g, dtype=torch.float32)


def _forward_backward(plan, x, out_numel, out_dtype):
    y = torch.empty(out_numel, dtype=out_dtype, device="cuda")
    plan.forward(x, y)
    z = torch.empty_like(x)
    plan.backward(y, z, 1)       # scale::full
    torch.cuda.synchronize()
    return y, z


def _c2c_case(gb, report, size, prec, tensor_cores, seed, ref=None):
    n = int(np.prod(size))
    box = gb.box3d((0, 0, 0), [s - 1 for s in size])
    plan = gb.fft3d(box, box)
    if tensor_cores:
        plan.set_tensor_cores(True)
    x = _complex_input(n, prec, seed)
    y, z = _forward_backward(plan, x, n, x.dtype)
    xh = x.cpu().numpy()
    del x
    if ref is None:
        ref = O.fft3d_c2c(xh, size)
    e_f = O.rel_l2(y.cpu().numpy(), ref)
    del y
    e_b = O.rel_l2(z.cpu().numpy(), xh)
    del z
    torch.cuda.empty_cache()
    form = "tensor cores" if tensor_cores else ("plain FP32" if prec == 0 else "FP64")
    report.append(f"c2c {size} {form}: forward rel-L2 {e_f:.3e} vs FP64 oracle, round trip {e_b:.3e}")
    assert e_f <= TOL[prec] and e_b <= TOL[prec], (e_f, e_b)
    assert gb.device_status() == 0
    return ref


def test_c2c_512cube_float_plain_and_tensor_cores(gb, report):
    ref = _c2c_case(gb, report, (512, 512, 512), 0, False, 512)
    _c2c_case(gb, report, (512, 512, 512), 0, True, 512, ref)


def test_c2c_1024x1024x512_float_plain_and_tensor_cores(gb, report):
    ref = _c2c_case(gb, report, (1024, 1024, 512), 0, False, 1024)
    _c2c_case(gb, report, (1024, 1024, 512), 0, True, 1024, ref)


def test_c2c_512cube_double(gb, report):
    _c2c_case(gb, report, (512, 512, 512), 1, False, 5120)


def test_r2c_512cube_float(gb, report):
    size = (512, 512, 512)
    n = int(np.prod(size))
    box = gb.box3d((0, 0, 0), [s - 1 for s in size])
    plan = gb.fft3d_r2c(box, box.r2c(0), 0)
    x = _real_input(n, 2512)
    y, z = _forward_backward(plan, x, plan.size_outbox(), torch.complex64)
    xh = x.cpu().numpy()
    e_f = O.rel_l2(y.cpu().numpy(), O.fft3d_r2c(xh, size, 0))
    e_b = O.rel_l2(z.cpu().numpy(), xh)
    report.append(f"r2c {size} float: forward rel-L2 {e_f:.3e} vs FP64 oracle, round trip {e_b:.3e}")
    assert e_f <= TOL[0] and e_b <= TOL[0], (e_f, e_b)
    assert gb.device_status() == 0


def test_dct2_256cube_float(gb, report):
    size = (256, 256, 256)
    n = int(np.prod(size))
    box = gb.box3d((0, 0, 0), [s - 1 for s in size])
    plan = gb.rtransform(gb.kind.cos, box, box)
    x = _real_input(n, 3256)
    y, z = _forward_backward(plan, x, n, torch.float32)
    xh = x.cpu().numpy()
    e_f = O.rel_l2(y.cpu().numpy(), O.rtransform(O.COS, xh, size))
    e_b = O.rel_l2(z.cpu().numpy(), xh)
    report.append(f"DCT-II {size} float: forward rel-L2 {e_f:.3e} vs FP64 oracle, round trip {e_b:.3e}")
    assert e_f <= TOL[0] and e_b <= TOL[0], (e_f, e_b)
    assert gb.device_status() == 0
