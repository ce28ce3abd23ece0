"""The surrogate's convolution on the tensor cores (hps_nn_conv_forward_tc:
tcgen05 BF16 MMA, FP32 accumulation in tensor memory, clusters splitting the
input channels) against the FP64 numpy oracle (oracle/nn_oracle.py) for
every layer of the network, at the test plane and at the 32 x 128 mesh the
shipped network runs on, and the shapes it refuses."""
import ctypes as C

import numpy as np
import pytest

from oracle import nn_oracle as N

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


def p(t):
    return C.c_void_p(t.data_ptr())


def run(entry, dims, x, w, b, relu, skip=None):
    from hpsim_gb300._capi import call
    B, ci, co, H, W, stride, up = (int(v) for v in dims)
    ho, wo = (H * up - 1) // stride + 1, (W * up - 1) // stride + 1
    X = torch.tensor(x, dtype=torch.bfloat16, device="cuda")
    Wt = torch.tensor(w, dtype=torch.bfloat16, device="cuda")
    Bt = torch.tensor(b, device="cuda")
    SK = None if skip is None else torch.tensor(skip, dtype=torch.bfloat16, device="cuda")
    Y = torch.empty((B, co, ho, wo), dtype=torch.bfloat16, device="cuda")
    call(entry, dims.ctypes.data_as(C.POINTER(C.c_int)), p(X), p(Wt), p(Bt), relu,
         None if SK is None else p(SK), p(Y), None)
    torch.cuda.synchronize()
    return Y.float().cpu().numpy()


@pytest.mark.parametrize("plane", [(2, 16, 8), (1, 128, 32), (3, 32, 16)])
@pytest.mark.parametrize("layer", range(10))
def test_tensor_core_layer_matches_oracle(layer, plane):
    from hpsim_gb300 import surrogate as S
    ci, co, stride, up, relu = S.ARCH[layer]
    B, H, W = plane
    rng = np.random.default_rng(100 * layer + H)
    dims = np.array([B, ci, co, H, W, stride, up], np.int32)
    x = N.bf16_round(rng.normal(size=(B, ci, H, W)).astype(np.float32))
    w = N.bf16_round((rng.normal(size=(co, ci, 3, 3)) / np.sqrt(9 * ci)).astype(np.float32))
    b = rng.normal(size=co).astype(np.float32) * 0.1
    y = run("hps_nn_conv_forward_tc", dims, x, w, b, relu)
    _, ref = N.conv_forward(x, w, b, stride, up, relu)
    # one BF16 rounding of an FP32 sum (the products of BF16 values are exact)
    assert np.all(np.abs(y - ref) <= 2.0 ** -7 * np.abs(ref) + 1e-5 * np.abs(ref).max())
    # against the CUDA-core kernel: the same up to the sums' order
    y_cc = run("hps_nn_conv_forward", dims, x, w, b, relu)
    assert np.all(np.abs(y - y_cc) <= 2.0 ** -7 * np.abs(y_cc) + 1e-5 * np.abs(y_cc).max())
    # the fused skip addition: the layer's BF16 output plus skip, rounded again
    sk = N.bf16_round(rng.normal(size=y.shape).astype(np.float32))
    y2 = run("hps_nn_conv_forward_tc", dims, x, w, b, relu, sk)
    assert np.array_equal(y2, N.bf16_round(y + sk))


def test_tensor_core_layer_refuses_shapes_it_does_not_take():
    from hpsim_gb300 import HPSim  # noqa: F401  (loads the library)
    rng = np.random.default_rng(0)
    for dims in ([1, 128, 192, 8, 8, 1, 1],   # c_out > 128
                 [1, 96, 32, 8, 8, 1, 1],     # c_in not a power of two
                 [1, 64, 32, 8, 7, 1, 1]):    # odd w_in
        d = np.array(dims, np.int32)
        x = rng.normal(size=(d[0], d[1], d[3], d[4])).astype(np.float32)
        w = rng.normal(size=(d[2], d[1], 3, 3)).astype(np.float32)
        with pytest.raises(Exception):
            run("hps_nn_conv_forward_tc", d, x, w, np.zeros(d[2], np.float32), 1)


def test_training_forward_on_tensor_cores_matches_cuda_cores():
    """Network.forward of a batch runs its layers on the tensor cores; the
    prediction equals the CUDA-core layers' to the BF16 activations'
    precision (2% in norm), and no pipeline wait gave up."""
    from hpsim_gb300 import surrogate as S
    net = S.Network(seed=7)
    rng = np.random.default_rng(7)
    x = torch.tensor(N.bf16_round(rng.normal(size=(4, 2, 128, 32)).astype(np.float32)), dtype=torch.bfloat16,
                     device="cuda")
    preds = {}
    for tc in (True, False):
        net.tensor_cores = tc
        preds[tc] = net.predict(x).cpu().numpy()
    assert net.tensor_core_errors() == 0
    assert np.linalg.norm(preds[True] - preds[False]) <= 0.02 * np.linalg.norm(preds[False])
