"""GPU: the network kernels of the learned near-singular quadrature
(gb_mlp.cu, include/gb_mlp.h) against the float64 reference network of the
oracle (oracle/lq.py): forward, loss gradient, one Adam step, and training on
labels of the reference's 64 x 64 fallback rule."""
import ctypes

import numpy as np
import pytest

from oracle import lq


def _lib():
    from bem3_emf_b2_gb300 import lib
    L = lib()
    vp, ci, cf = ctypes.c_void_p, ctypes.c_int, ctypes.c_float
    L.gb_mlp_create.argtypes = [ci, vp, vp]
    L.gb_mlp_create.restype = ci
    L.gb_mlp_destroy.argtypes = [vp]
    L.gb_mlp_destroy.restype = None
    L.gb_mlp_param_count.argtypes = [vp]
    L.gb_mlp_param_count.restype = ctypes.c_size_t
    L.gb_mlp_set_params.argtypes = [vp, vp]
    L.gb_mlp_get_params.argtypes = [vp, vp]
    L.gb_mlp_forward_host.argtypes = [vp, ci, vp, vp]
    L.gb_mlp_loss_grad_host.argtypes = [vp, ci, vp, vp, vp, vp]
    L.gb_mlp_train_host.argtypes = [vp, ci, vp, vp, ci, ci, cf, vp]
    for n in ("gb_mlp_set_params", "gb_mlp_get_params", "gb_mlp_forward_host", "gb_mlp_loss_grad_host",
              "gb_mlp_train_host"):
        getattr(L, n).restype = ci
    return L


class Net:
    def __init__(self, widths, params):
        from bem3_emf_b2_gb300 import last_error
        self.L = _lib()
        self.err = last_error
        w = np.array(widths, np.int32)
        h = ctypes.c_void_p()
        assert self.L.gb_mlp_create(len(widths) - 1, w.ctypes.data, ctypes.byref(h)) == 0, last_error()
        self.h = h
        self.widths = widths
        assert self.L.gb_mlp_param_count(h) == params.size
        self.set(params)

    def set(self, params):
        p = np.ascontiguousarray(params, np.float32)
        assert self.L.gb_mlp_set_params(self.h, p.ctypes.data) == 0, self.err()

    def get(self):
        p = np.zeros(self.L.gb_mlp_param_count(self.h), np.float32)
        assert self.L.gb_mlp_get_params(self.h, p.ctypes.data) == 0, self.err()
        return p

    def forward(self, X):
        X = np.ascontiguousarray(X, np.float32)
        Y = np.zeros((X.shape[0], self.widths[-1]), np.float32)
        assert self.L.gb_mlp_forward_host(self.h, X.shape[0], X.ctypes.data, Y.ctypes.data) == 0, self.err()
        return Y

    def loss_grad(self, X, T):
        X = np.ascontiguousarray(X, np.float32)
        T = np.ascontiguousarray(T, np.float32)
        g = np.zeros(self.L.gb_mlp_param_count(self.h), np.float32)
        loss = ctypes.c_double()
        assert self.L.gb_mlp_loss_grad_host(self.h, X.shape[0], X.ctypes.data, T.ctypes.data, ctypes.byref(loss),
                                            g.ctypes.data) == 0, self.err()
        return loss.value, g

    def train(self, X, T, B, steps, lr):
        X = np.ascontiguousarray(X, np.float32)
        T = np.ascontiguousarray(T, np.float32)
        losses = np.zeros(steps)
        assert self.L.gb_mlp_train_host(self.h, X.shape[0], X.ctypes.data, T.ctypes.data, B, steps, lr,
                                        losses.ctypes.data) == 0, self.err()
        return losses

    def close(self):
        self.L.gb_mlp_destroy(self.h)


def _data(n, seed):
    c, rt, k = lq.sample_pairs(n, seed)
    X, h = lq.features(c, rt, k)
    return X.astype(np.float32), lq.targets(lq.labels(c, rt, k, 3), h).astype(np.float32)


@pytest.mark.gpu
def test_forward_and_gradient_match_the_reference(gb_build):
    ps = lq.init_params(1)
    ps = [(W, (0.05 * np.arange(b.size) / b.size).astype(np.float32)) for W, b in ps]
    params = lq.pack(ps)
    X, T = _data(1000, 2)
    net = Net(lq.WIDTHS, params)
    Y = net.forward(X)
    Yr, _ = lq.mlp_forward(ps, X.astype(np.float64))
    ef = np.linalg.norm(Y - Yr) / np.linalg.norm(Yr)
    loss, g = net.loss_grad(X, T)
    lr_, grads = lq.mlp_loss_grad(ps, X.astype(np.float64), T.astype(np.float64))
    gr = lq.pack([(gw, gb) for gw, gb in grads])
    net.close()
    assert ef <= 1e-5, ef
    assert abs(loss - lr_) <= 1e-5 * lr_, (loss, lr_)
    for li, (Wg, bg) in enumerate(lq.unpack(g)):
        Wr, br = grads[li]
        assert np.linalg.norm(Wg - Wr) <= 1e-4 * np.linalg.norm(Wr), ("W", li, np.linalg.norm(Wg - Wr) / np.linalg.norm(Wr))
        assert np.linalg.norm(bg - br) <= 1e-4 * np.linalg.norm(br), ("b", li)
    assert np.linalg.norm(g - gr) <= 1e-4 * np.linalg.norm(gr)


@pytest.mark.gpu
def test_adam_step_and_training(gb_build):
    ps = lq.init_params(3)
    p0 = lq.pack(ps)
    X, T = _data(4096, 4)
    Xv, Tv = _data(1024, 5)
    net = Net(lq.WIDTHS, p0)
    # one Adam step from zero moments: p - lr * g / (|g| + eps) elementwise
    lr = 1e-3
    _, g = net.loss_grad(X[:512], T[:512])
    net.train(X[:512], T[:512], 512, 1, lr)
    p1 = net.get()
    expect = p0 - lr * g / (np.abs(g) + 1e-8)
    assert np.abs(p1 - expect).max() <= 1e-6 + 1e-4 * lr, np.abs(p1 - expect).max()
    # training on the 64 x 64 rule's labels lowers the held-out loss
    net.set(p0)
    v0, _ = net.loss_grad(Xv, Tv)
    losses = net.train(X, T, 512, 400, 1e-3)
    v1, _ = net.loss_grad(Xv, Tv)
    net.close()
    print("held-out loss %.3e -> %.3e after 400 steps (training batch %.3e -> %.3e)" %
          (v0, v1, losses[:8].mean(), losses[-8:].mean()))
    assert np.all(np.isfinite(losses))
    assert v1 <= 0.2 * v0, (v0, v1)
