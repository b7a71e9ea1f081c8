"""Host-side argument checks of the learned-quadrature entry points
(include/gb_bem.h gb_lq_*): no GPU work is reached."""
import ctypes

import pytest


def _lib(gb_build):
    from bem3_emf_b2_gb300 import lib
    L = lib()
    L.gb_lq_enable.argtypes = [ctypes.c_int, ctypes.c_double]
    L.gb_lq_train.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_float, ctypes.c_uint, ctypes.c_void_p]
    L.gb_last_error.restype = ctypes.c_char_p
    return L


def test_enable_needs_a_trained_network(gb_build):
    L = _lib(gb_build)
    assert L.gb_lq_enable(1, 1e-7) != 0
    assert b"no trained network" in L.gb_last_error()
    assert L.gb_lq_enable(0, 0.0) != 0
    assert L.gb_lq_enable(0, 1e-7) == 0


def test_train_needs_collected_pairs(gb_build):
    L = _lib(gb_build)
    info = (ctypes.c_double * 5)()
    assert L.gb_lq_train(2, 1024, 1e-3, 1, info) != 0
    assert b"collected pairs" in L.gb_last_error()
