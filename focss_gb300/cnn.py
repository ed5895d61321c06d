"""Convolutional correction of the learned-DBP output (focss_cnn_*): a 4-layer
1D CNN (64 channels, kernel 9) on [Re y, Im y] and first-order perturbation
triplets of y (T(m, n) + T(-m, -n), SINO::term, src/focss/equalizer/
sino.cpp:161-171), whose output is added back to the symbols.  Training
(forward, backward, Adam) runs on the GPU."""
from __future__ import annotations

import ctypes as C

import numpy as np

from ._lib import check, lib
from .api import Context, Field

P = C.c_void_p
LAYERS = ((16, 64), (64, 64), (64, 64), (64, 16))  # (cin, cout), padded
KW = 9


def layout():
    """[(w_offset, w_shape, b_offset, cout)] of the flat parameter vector."""
    out, o = [], 0
    for cin, cout in LAYERS:
        out.append((o, (cout, KW, cin), o + cout * KW * cin, cout))
        o += cout * KW * cin + cout
    return out, o


# Triplet offsets (m, n) of the input features: the SPM term and the
# neighbours along n = 0 and m = n, m = -n that dominate first-order
# perturbation coefficients.
TRIPLETS = ((0, 0), (0, 1), (0, 2), (0, 3), (1, 1), (1, -1), (1, 2))


def he_init(rng, zero_last=True, n_triplets=0, last_scale=1.0):
    """He-normal weights, zero biases; the unused input channels of layer 1 and
    output channels of layer 4 zero; layer 4 zero (zero_last: the network
    starts as the identity z = y) or scaled by last_scale."""
    lay, total = layout()
    p = np.zeros(total, np.float32)
    used = 2 + 2 * n_triplets  # input channels in use in layer 1
    fan = [used * KW, 64 * KW, 64 * KW, 64 * KW]
    for l, (wo, shape, bo, cout) in enumerate(lay):
        w = rng.standard_normal(shape) * np.sqrt(2.0 / fan[l])
        if l == 0:
            w[:, :, used:] = 0
        if l == 3:
            w[2:] = 0
            w *= 0.0 if zero_last else last_scale
        p[wo:wo + w.size] = w.ravel()
    return p


class CorrectionCNN:
    def __init__(self, length, batch, input_scale, ctx=None, triplets=()):
        self.ctx = ctx or Context.default()
        self.length, self.batch = length, batch
        h = C.c_void_p()
        check(lib().focss_cnn_create(self.ctx.h, 64, KW, length, batch, input_scale, C.byref(h)), self.ctx.h)
        self.h = h
        self.n_params = lib().focss_cnn_num_params(h)
        self.triplets = tuple(triplets)
        if self.triplets:
            m = np.array([t[0] for t in self.triplets], np.int32)
            n = np.array([t[1] for t in self.triplets], np.int32)
            check(lib().focss_cnn_set_triplets(h, len(self.triplets), m.ctypes.data_as(P), n.ctypes.data_as(P)),
                  self.ctx.h)

    def set_params(self, flat):
        f = np.ascontiguousarray(flat, np.float32)
        check(lib().focss_cnn_set_params(self.h, f.ctypes.data_as(P), f.size), self.ctx.h)

    def get_params(self):
        p = np.zeros(self.n_params, np.float32)
        g = np.zeros(self.n_params, np.float32)
        check(lib().focss_cnn_get_params(self.h, p.ctypes.data_as(P), g.ctypes.data_as(P), p.size), self.ctx.h)
        return p, g

    def forward(self, y: Field) -> Field:
        z = Field(y.domain, batch=y.batch, ctx=self.ctx)
        check(lib().focss_cnn_forward(self.h, y.h, z.h), self.ctx.h)
        return z

    def loss_grad(self, y: Field, tx: Field) -> float:
        loss = C.c_double()
        check(lib().focss_cnn_loss_grad(self.h, y.h, tx.h, C.byref(loss)), self.ctx.h)
        return loss.value

    def adam_step(self, lr=1e-3, beta1=0.9, beta2=0.999, eps=1e-8):
        check(lib().focss_cnn_adam_step(self.h, lr, beta1, beta2, eps), self.ctx.h)

    def identity_params(self, flat):
        """flat with layer 4 zeroed: the network then passes y through."""
        p = np.array(flat, np.float32)
        lay, _ = layout()
        wo, shape, bo, cout = lay[3]
        p[wo:bo + cout] = 0
        return p

    def fit(self, y: Field, tx: Field, iters=100, lr=1e-3):
        hist = []
        for _ in range(iters):
            hist.append(self.loss_grad(y, tx))
            self.adam_step(lr)
        return hist

    def close(self):
        from ._lib import alive
        if getattr(self, "h", None) and alive():
            lib().focss_cnn_destroy(self.h)
        self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
