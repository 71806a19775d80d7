"""Host-side mirror of the reference's NeuralRadianceCache (renderer/network_interface.h:8-31)
over the C ABI in include/rtc8_nrc.h.

    cache = NeuralRadianceCache()
    cache.initialize(PositionEncoding.HashGrid, num_hidden_layers=2, learning_rate=1e-2)
    cache.infer(stream, input_ptr, n, prediction_ptr)
    cache.train(stream, input_ptr, target_ptr, n)      # loss=True returns the batch loss (syncs)
    cache.finalize()

Pointers are device addresses (ints) or CUDA tensors; inputs are AoS RadianceQuery records of
14 floats, predictions and targets 3 floats per record, as in the reference.
"""
from __future__ import annotations

import ctypes as C
import enum

import numpy as np

from . import _lib
from ._lib import NrcConfig

NRC_ENCODING_REFERENCE = 0
NRC_ENCODING_VOLUME = 1
NRC_ENCODING_HASHGRID = 2
NRC_OUTPUT_NONE = 0
NRC_OUTPUT_EXP = 1


class PositionEncoding(enum.IntEnum):
    """network_interface.h:8-11: TriangleWave -> NRC_ENCODING_REFERENCE, HashGrid (the
    reference's default, renderer_scene.cpp:50) -> NRC_ENCODING_HASHGRID."""
    TriangleWave = 0
    HashGrid = 1


class NrcError(RuntimeError):
    pass


def _ptr(x) -> int:
    if x is None:
        return 0
    if isinstance(x, int):
        return x
    return int(x.data_ptr())


def _check(rc: int, what: str) -> None:
    if rc != 0:
        msg = _lib.load().nrc_last_error()
        raise NrcError(f"{what} failed with code {rc}: {msg.decode() if msg else ''}")


def default_config(encoding: int) -> NrcConfig:
    cfg = NrcConfig()
    _lib.load().nrc_default_config(encoding, C.byref(cfg))
    return cfg


class NeuralRadianceCache:
    def __init__(self):
        self.lib = _lib.load()
        self.h = None

    # network_interface.h:25 initialize(PositionEncoding, numHiddenLayers, learningRate)
    def initialize(self, pos_encoding: PositionEncoding = PositionEncoding.TriangleWave, num_hidden_layers: int = 2,
                   learning_rate: float = 1e-2, config: NrcConfig | None = None) -> None:
        if config is None:
            config = default_config(NRC_ENCODING_HASHGRID if pos_encoding == PositionEncoding.HashGrid
                                    else NRC_ENCODING_REFERENCE)
            config.num_hidden_layers = num_hidden_layers
            config.learning_rate = learning_rate
        self.config = config
        h = C.c_void_p()
        _check(self.lib.nrc_create(C.byref(config), C.byref(h)), "nrc_create")
        self.h = h

    def finalize(self) -> None:
        if self.h:
            self.lib.nrc_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.finalize()
        except Exception:
            pass

    def infer(self, stream, input_data, num_data: int, prediction_data) -> None:
        _check(self.lib.nrc_infer(self.h, C.c_void_p(_ptr(stream)), C.c_void_p(_ptr(input_data)), num_data,
                                  C.c_void_p(_ptr(prediction_data))), "nrc_infer")

    def infer_indexed(self, stream, input_data, index, count, max_count: int, prediction_data) -> None:
        """nrc_infer_indexed: inference on the records index[0 .. *count) (device tensors; count
        holds one uint32 on the device), leaving the other records of prediction_data as they are."""
        _check(self.lib.nrc_infer_indexed(self.h, C.c_void_p(_ptr(stream)), C.c_void_p(_ptr(input_data)),
                                          C.c_void_p(_ptr(index)), C.c_void_p(_ptr(count)), max_count,
                                          C.c_void_p(_ptr(prediction_data))), "nrc_infer_indexed")

    def train(self, stream, input_data, target_data, num_data: int, loss: bool = False):
        out = C.c_float(0.0)
        _check(self.lib.nrc_train(self.h, C.c_void_p(_ptr(stream)), C.c_void_p(_ptr(input_data)),
                                  C.c_void_p(_ptr(target_data)), num_data, C.byref(out) if loss else None),
               "nrc_train")
        return out.value if loss else None

    def encode(self, stream, input_data, num_data: int, out) -> None:
        _check(self.lib.nrc_encode(self.h, C.c_void_p(_ptr(stream)), C.c_void_p(_ptr(input_data)), num_data,
                                   C.c_void_p(_ptr(out))), "nrc_encode")

    def layout(self) -> dict:
        L = C.c_int32()
        ins = (C.c_int32 * 8)()
        outs = (C.c_int32 * 8)()
        tot = C.c_int64()
        _check(self.lib.nrc_get_layout(self.h, C.byref(L), ins, outs, C.byref(tot)), "nrc_get_layout")
        return {"L": L.value, "in": list(ins)[: L.value], "out": list(outs)[: L.value], "total": tot.value}

    def params(self) -> np.ndarray:
        out = np.empty(self.layout()["total"], np.float32)
        _check(self.lib.nrc_get_params(self.h, _lib.ptr(out, C.c_float)), "nrc_get_params")
        return out

    def set_params(self, p: np.ndarray) -> None:
        p = np.ascontiguousarray(p, np.float32)
        _check(self.lib.nrc_set_params(self.h, _lib.ptr(p, C.c_float)), "nrc_set_params")

    def gradients(self) -> np.ndarray:
        out = np.empty(self.layout()["total"], np.float32)
        _check(self.lib.nrc_get_gradients(self.h, _lib.ptr(out, C.c_float)), "nrc_get_gradients")
        return out

    def device_errors(self) -> int:
        return int(self.lib.nrc_device_errors(self.h))


def selftest_mma_rate(n: int, count: int = 1024) -> float:
    """nrc_selftest_mma_rate: SM cycles per back-to-back M = 128 x N = n x K = 16 FP16 MMA issued by
    one thread (the rate the MLP kernels' layer shapes can reach)."""
    lib = _lib.load()
    c = C.c_double(0.0)
    _check(lib.nrc_selftest_mma_rate(n, count, C.byref(c)), "nrc_selftest_mma_rate")
    return c.value


def selftest_mma(a: np.ndarray, b: np.ndarray, a_mode: int, b_mode: int) -> np.ndarray:
    a = np.ascontiguousarray(a, np.float32)
    b = np.ascontiguousarray(b, np.float32)
    d = np.zeros((128, 64), np.float32)
    lib = _lib.load()
    _check(lib.nrc_selftest_mma(_lib.ptr(a, C.c_float), _lib.ptr(b, C.c_float), a_mode, b_mode,
                                _lib.ptr(d, C.c_float)), "nrc_selftest_mma")
    return d
