"""The tcgen05 inference kernel of the surrogate's network against an FP64 reference
and against the warp-level mma.sync kernel.

Inference (pt_mlp_predict*) runs every layer on tcgen05.mma: BF16 operands in shared
memory, FP32 accumulation in tensor memory, bias + GELU on the accumulator read back
with tcgen05.ld.  The reference is the same network in FP64 with the weights, inputs
and hidden activations rounded to BF16 where the kernel rounds them, and GELU in the
same tanh form with an exact tanh (the kernels use the hardware tanh); the tolerance
covers the FP32 summation order and that approximation, far below one BF16 step of
the outputs."""
import numpy as np
import pytest

from pandemicthrust_gb300 import surrogate as sg

pytestmark = pytest.mark.gpu


C0, C1 = np.sqrt(2 / np.pi), np.sqrt(2 / np.pi) * 0.044715   # GELU, tanh form


def bf16(x):
    u = np.ascontiguousarray(x, np.float32).view(np.uint32).astype(np.uint64)
    u = ((u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000).astype(np.uint32)
    return u.view(np.float32).astype(np.float64)


def reference_forward(params, widths, X):
    """FP64 forward; weights, inputs and hidden activations rounded to BF16."""
    H, off = bf16(X), 0
    L = len(widths) - 1
    for l in range(L):
        n = widths[l + 1] * widths[l]
        W = bf16(params[off:off + n]).reshape(widths[l + 1], widths[l])
        off += n
        b = params[off:off + widths[l + 1]].astype(np.float64)
        off += widths[l + 1]
        Z = H @ W.T + b
        H = bf16(0.5 * Z * (1 + np.tanh(Z * (C0 + C1 * Z * Z)))) if l + 1 < L else Z
    return H


@pytest.mark.parametrize("widths,rows", [([11, 256, 256, 256, 256, 222], 1000),   # the surrogate's shape
                                          ([11, 256, 256, 256, 256, 222], 128),
                                          ([16, 64, 32], 300),
                                          ([40, 128, 256, 96], 4100),
                                          ([160, 192, 48], 777)])   # K stages of 80 + 80 and 128 + 64
def test_tcgen05_forward_matches_reference_and_mma_sync(native_lib, widths, rows):
    rng = np.random.default_rng(11)
    net = sg.MLP(widths, max_batch=4096, seed=5)
    p = net.get_params()
    # non-zero biases so the epilogue's bias add is checked
    p = p + rng.standard_normal(p.shape).astype(np.float32) * 0.05
    net.set_params(p)
    X = rng.uniform(-1, 1, (rows, widths[0])).astype(np.float32)
    net.set_tcgen05(True)
    y_tc = net.predict(X)
    net.set_tcgen05(False)
    y_mma = net.predict(X)
    net.close()
    ref = reference_forward(p, widths, X)
    scale = np.abs(ref).max()
    # both kernels accumulate in FP32; the hidden activations are BF16 in all three
    assert np.abs(y_tc - ref).max() <= 2e-2 * scale
    assert np.abs(y_tc - ref).mean() <= 2e-3 * scale
    assert np.abs(y_tc - y_mma).mean() <= 2e-3 * scale
    assert np.isfinite(y_tc).all()


def test_tcgen05_ensemble_on_device_buffers_equals_host_path(native_lib):
    torch = pytest.importorskip("torch")
    s = sg.Surrogate(1_000_000, seed=3, members=2, max_batch=512)
    X = sg.features(sg.sample_scenarios(1500, np.random.default_rng(4)))
    y_host = s.raw_features(X)
    xd = torch.from_numpy(X).cuda()
    yd = torch.zeros((len(X), sg.OUTPUTS), dtype=torch.float32, device="cuda")
    torch.cuda.synchronize()
    s.raw_device(xd.data_ptr(), len(X), yd.data_ptr())
    torch.cuda.synchronize()
    np.testing.assert_array_equal(yd.cpu().numpy(), y_host)
    s.close()


def test_ensemble_mean_layer_equals_the_mean_of_the_members(native_lib):
    """An ensemble runs its members' last layers as one GEMM over their concatenated
    activations (k_umma_mean_layer).  Its output equals the mean of the members' own
    predictions up to FP32 summation order: the hidden layers are the same kernels."""
    rng = np.random.default_rng(21)
    s = sg.Surrogate(1_000_000, seed=5, members=4, max_batch=2048)
    for net in s.nets:
        p = net.get_params()
        net.set_params(p + rng.standard_normal(p.shape).astype(np.float32) * 0.05)
    X = sg.features(sg.sample_scenarios(3000, rng))   # two chunks, the second a partial tile
    y = s.raw_features(X)
    each = np.mean([net.predict(X) for net in s.nets], axis=0)
    s.close()
    scale = np.abs(each).max()
    assert np.isfinite(y).all()
    assert np.abs(y - each).max() <= 1e-5 * scale
