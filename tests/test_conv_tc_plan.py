"""The tensor-core convolution's launch plan, host side (no GPU): the weight
tile sizes hps_nn_conv_tc_tile_bytes reports for the surrogate network's
layers, and the shapes the kernel refuses.

A layer's tiles hold, per cluster rank, its K = 9 taps x (its share of the
input channels) in chunks of 64 BF16 values, each chunk one 128-byte row per
output channel padded to a multiple of 16 channels (the MMA's N)."""
import ctypes as C

import numpy as np
import pytest


@pytest.fixture(scope="module")
def tile_bytes():
    from hpsim_gb300 import build
    build.build()
    from hpsim_gb300._capi import call

    def f(dims):
        d = np.ascontiguousarray(dims, np.int32)
        nb = C.c_uint64()
        call("hps_nn_conv_tc_tile_bytes", d.ctypes.data_as(C.POINTER(C.c_int)), C.byref(nb))
        return nb.value
    return f


@pytest.mark.parametrize("batch", [1, 8, 32])
@pytest.mark.parametrize("plane", [(128, 32), (256, 64)])
def test_every_layer_of_the_network_has_tensor_core_tiles(tile_bytes, batch, plane):
    from hpsim_gb300 import surrogate as S
    for dims in S.layer_shapes(batch, *plane):
        ci, co = int(dims[1]), int(dims[2])
        nb = tile_bytes(dims)
        assert nb > 0, dims
        row = (co + 15) // 16 * 16 * 128  # one K chunk: 64 BF16 values per padded output channel
        assert nb % row == 0
        k_padded = nb // row * 64
        # every (tap, channel) pair has a K slot; the padding is less than
        # one chunk per cluster rank (at most 8 ranks)
        assert 0 <= k_padded - 9 * ci < 8 * 64, (dims, nb)


def test_shapes_the_kernel_does_not_take_have_no_tiles(tile_bytes):
    assert tile_bytes([1, 128, 192, 8, 8, 1, 1]) == 0  # c_out > 128
    assert tile_bytes([1, 96, 32, 8, 8, 1, 1]) == 0    # c_in not a power of two
    assert tile_bytes([1, 64, 32, 8, 7, 1, 1]) == 0    # odd w_in
    assert tile_bytes([1, 64, 32, 8, 8, 1, 1]) > 0


def test_malformed_layer_shapes_are_rejected(tile_bytes):
    for dims in ([1, 64, 32, 8, 8, 3, 1],    # stride 3
                 [1, 64, 32, 8, 8, 1, 3],    # upsampling 3
                 [1, 1024, 32, 8, 8, 1, 1],  # more input channels than a layer takes
                 [0, 64, 32, 8, 8, 1, 1]):   # empty batch
        with pytest.raises(Exception):
            tile_bytes(dims)
