"""The no-allocation variant of the metric product, rs_metric_apply_device_noalloc, called
through the C ABI. It exists for callers that cannot allocate device memory while a product
runs (a host whose device memory is held by its own pool after set-up, or a latency-critical
stream, since cudaMalloc and cudaFree can synchronize the device).

* On a freshly built metric, before any regular product has reserved that metric's buffers,
  two no-alloc calls in a row leave the device's free memory unchanged (cudaMemGetInfo), and
  both give the product of the regular device entry point rs_metric_apply_device on the same
  input (the same kernels in the same order, so the tolerance below is loose for what is
  expected to be equal bit for bit).
* A product whose scratch would exceed the fixed 64 MiB is refused with InvalidOption.

Collected last on purpose; it also passes alone in a fresh process, where its first call does
the scratch set-up."""
import ctypes as C

import numpy as np
import pytest

import golden_io as G
import rs_gb300 as R
from rs_gb300 import generators as gen

pytestmark = pytest.mark.gpu

TOL = 1e-12


def _noalloc(m, x, y, nb, w_hi=1.0, w_lo=1.0):
    code = R.load_library().rs_metric_apply_device_noalloc(m._h, w_hi, w_lo, nb, C.c_void_p(x.data_ptr()),
                                                           C.c_void_p(y.data_ptr()))
    if code != 0:
        L = R.load_library()
        raise R.RsError(code, L.rs_last_error_kind().decode(), L.rs_last_error_operation().decode(),
                        L.rs_last_error().decode())


@pytest.mark.parametrize("nb", [1, 2, 4])
def test_noalloc_product_matches_the_device_entry_point(nb):
    torch = pytest.importorskip("torch")
    ctx = R.Context(0)
    P, F = gen.config_c2(level=4)
    x = torch.from_numpy(np.random.default_rng(11).standard_normal((nb, 3 * len(P)))).cuda()
    y_ref = torch.zeros_like(x)
    y1 = torch.full_like(x, float("nan"))
    y2 = torch.full_like(x, float("nan"))
    # the kernels of the product loaded once (lazy module loading may place their code on first
    # use), on another metric of the same mesh
    warm = R.FaceMetricTree(F, P, R.Exponents(), R.ClusterTreeOptions(), ctx)
    _noalloc(warm, x, y1, nb, 1.0, 0.7)
    m = R.FaceMetricTree(F, P, R.Exponents(), R.ClusterTreeOptions(), ctx)
    ctx.synchronize()
    torch.cuda.synchronize()
    free0 = torch.cuda.mem_get_info()[0]
    _noalloc(m, x, y1, nb, 1.0, 0.7)
    _noalloc(m, x, y2, nb, 1.0, 0.7)
    ctx.synchronize()
    assert torch.cuda.mem_get_info()[0] == free0  # nothing allocated by the two calls
    m.apply_device(x.data_ptr(), y_ref.data_ptr(), nb, 1.0, 0.7)
    ctx.synchronize()
    ref = y_ref.cpu().numpy()
    assert np.all(np.isfinite(ref))
    for y in (y1, y2):
        assert G.normwise(y.cpu().numpy(), ref) <= TOL


def test_noalloc_refuses_more_than_its_scratch():
    torch = pytest.importorskip("torch")
    ctx = R.Context(0)
    P, F = gen.config_c2()  # 81,920 faces: three vectors need more than 64 MiB
    m = R.FaceMetricTree(F, P, R.Exponents(), R.ClusterTreeOptions(), ctx)
    x = torch.zeros((3, 3 * len(P)), dtype=torch.float64, device="cuda")
    y = torch.zeros_like(x)
    torch.cuda.synchronize()
    with pytest.raises(R.RsError) as e:
        _noalloc(m, x, y, 3)
    assert e.value.kind == "InvalidOption" and "64 MiB" in str(e.value)
    # one vector fits, and gives the regular product
    y_ref = torch.zeros_like(x[:1])
    m.apply_device(x[:1].data_ptr(), y_ref.data_ptr(), 1)
    _noalloc(m, x[:1], y[:1], 1)
    ctx.synchronize()
    assert torch.equal(y[:1], y_ref)
