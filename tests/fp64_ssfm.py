"""FP64 split-step restatement on the GPU (torch.fft, complex128) for the
full-size precision tests.

The C oracle (oracle/focss_oracle.c) takes minutes per link at N = 2^19 and
tens of thousands of steps on one host thread; this restatement runs the same
loops in complex128 on the device in seconds.  It follows the ADAPTIVE loop of
src/focss/solver/ssfm.cpp:92-118 (Strang steps L(h/2) N(h) L(h/2), the step
estimate of :136-140 from the peak power after the Kerr step, the remainder
as the last step), with the dispersion cache of :39-60 (omega_k in FFT order,
Nyquist bin positive), linear steps as :152-158 (loss exp(-alpha h/2) times
exp(i beta2/2 h omega^2) on the 1/N-normalized spectrum, field.cpp:343-352)
and the Kerr step of :160-164 (total power over modes times kappa gamma h).
Consecutive half steps L(h_i/2) L(h_{i+1}/2) are applied as one factor, which
is the same operator in exact arithmetic.  It is test infrastructure: the
tests pin it against the C oracle at small sizes before using it.
"""
from __future__ import annotations

import math

import torch


def _omega2(n, dt, device):
    i = torch.arange(n, dtype=torch.float64, device=device)
    i = torch.where(i <= n // 2, i, i - n)
    w = i * (2.0 * math.pi / (dt * n))
    return w * w


class _Loop:
    def __init__(self, x, dt, fiber, direction):
        self.n = x.shape[-1]
        self.w2 = _omega2(self.n, dt, x.device)
        self.f = fiber
        self.dir = direction
        self.spec = torch.fft.fft(x, dim=-1) / self.n

    def linear(self, step):
        # exp(-alpha step/2) * exp(i beta2/2 step w^2)
        g = math.exp(-0.5 * self.f.alpha * step)
        ph = (0.5 * self.f.beta2 * step) * self.w2
        self.spec *= torch.polar(torch.full_like(ph, g), ph)

    def kerr(self, step):
        a = torch.fft.ifft(self.spec, dim=-1) * self.n
        p = (a.real * a.real + a.imag * a.imag).sum(dim=0, keepdim=True)
        a *= torch.polar(torch.ones_like(p), (self.f.kappa * self.f.gamma * step) * p)
        return a, p

    def finish(self):
        return torch.fft.ifft(self.spec, dim=-1) * self.n


def run_steps(x, dt, fiber, h, direction=1.0):
    """Propagate x (complex128 tensor, modes x samples) over the step sizes h."""
    lp = _Loop(x, dt, fiber, direction)
    d = direction
    h = [float(v) for v in h]
    lp.linear(0.5 * h[0] * d)
    for i, step in enumerate(h):
        a, _ = lp.kerr(step * d)
        lp.spec = torch.fft.fft(a, dim=-1) / lp.n
        nxt = h[i + 1] if i + 1 < len(h) else 0.0
        lp.linear(0.5 * (step + nxt) * d)
    return lp.finish()


def run_adaptive(x, dt, fiber, max_phase, max_step, direction=1.0):
    """Free-running ADAPTIVE run (ssfm.cpp:92-118); returns (field, step sizes taken)."""
    lp = _Loop(x, dt, fiber, direction)
    d = direction
    arg = abs(fiber.kappa * fiber.gamma)

    def estimate(peak):
        h = max_phase / (arg * peak)
        return max_step if max_step < h else h

    step = estimate(float((x.real * x.real + x.imag * x.imag).sum(dim=0).max()))
    distance, taken = 0.0, []
    while distance + step < fiber.length:
        lp.linear(0.5 * step * d)
        a, p = lp.kerr(step * d)
        nxt = estimate(float(p.max()))
        lp.spec = torch.fft.fft(a, dim=-1) / lp.n
        lp.linear(0.5 * step * d)
        taken.append(step)
        distance += step
        step = nxt
    step = fiber.length - distance
    lp.linear(0.5 * step * d)
    a, _ = lp.kerr(step * d)
    lp.spec = torch.fft.fft(a, dim=-1) / lp.n
    lp.linear(0.5 * step * d)
    taken.append(step)
    return lp.finish(), taken
