"""End-to-end link helpers on the GPU: WDM 16QAM transmitter, amplified SSMF
propagation, centre-channel receiver, plain DBP and learned DBP scoring.

These follow the reference's experiment drivers (src/tasks/wdm_run.cpp:79-155,
src/tasks/sp_run.cpp:10-53, src/tasks/systems.cpp) with the benchmark
configurations' parameters; every step is a call into libfocss_gpu.
"""
from __future__ import annotations

import time
from dataclasses import dataclass

import numpy as np

from . import dsp
from .api import (Amplifier, Domain, Fiber, Field, SSFM, backward_propagation, cd_compensation, db_to_linear,
                  db_to_natural, dbm_to_watts, disp_to_beta2, span_loop)

LIGHT_SPEED = 299792458.0


@dataclass
class Link:
    spans: int = 20
    span_m: float = 80e3
    alpha_db_km: float = 0.2
    dispersion: float = 17e-6     # s/m^2 (17 ps/nm/km)
    gamma: float = 1.3e-3         # 1/W/m
    wavelength: float = 1.55e-6
    noise_figure_db: float = 5.0
    max_phase: float = 0.005
    max_step: float = 1000.0
    baud: float = 32e9
    channels: int = 5
    spacing: float = 50e9
    osf: int = 16
    roll_off: float = 0.1

    def fiber(self):
        return Fiber(db_to_natural(self.alpha_db_km * 1e-3), disp_to_beta2(self.dispersion, self.wavelength),
                     self.gamma, self.span_m, self.wavelength, 1.0)

    def gain(self):
        return db_to_linear(self.alpha_db_km * self.span_m / 1e3)

    def f0(self):
        return LIGHT_SPEED / self.wavelength


def wdm_transmitter(link: Link, n_symbols, batch, power_dbm, seed, ctx=None):
    """Per realization: `channels` independent 16QAM sequences, RRC shaped at
    `osf` samples/symbol and multiplexed (wdm_run.cpp:89-100).  Returns the
    field (batch realizations) and the centre channel's symbols."""
    p = np.sqrt(dbm_to_watts(power_dbm))
    rng = np.random.default_rng(seed)
    codes = rng.integers(0, 16, (batch * link.channels, 1, n_symbols))
    sym = dsp.qam16_map(codes, Domain(1, n_symbols, 1 / link.baud), batch=batch * link.channels, ctx=ctx)
    sym *= p
    shaped = dsp.rrc_shaping(sym, link.osf, link.roll_off)
    dt = shaped.domain.time_step
    n = shaped.domain.samples
    out = Field(Domain(1, n, dt, link.f0()), batch=batch, ctx=ctx)
    for b in range(batch):
        mux = dsp.wdm_mux(shaped.slice(b * link.channels, link.channels), link.spacing)
        out.copy_realizations(b, mux, 0, 1)
    centre = codes.reshape(batch, link.channels, n_symbols)[:, link.channels // 2]
    tx = dsp.qam16_map(centre[:, None, :], Domain(1, n_symbols, 1 / link.baud), batch=batch, ctx=ctx)
    tx *= p
    return out, tx


def propagate(link: Link, field: Field, seed=1):
    """forward_propagation (systems.cpp:39-56) with ADAPTIVE steps and ASE; returns total steps."""
    s = SSFM(link.fiber())
    s.set_grid(SSFM.ADAPTIVE)
    s.set_maximum_phase_shift(link.max_phase)
    s.set_maximum_step_size(link.max_step)
    amp = Amplifier(link.gain(), db_to_linear(link.noise_figure_db), seed=seed)
    steps = 0
    for i in range(link.spans):
        steps += int(s.run(field).sum())
        amp.amplify(field, counter=i)
    return steps


def centre_channel(link: Link, field: Field, dbp_osf=2):
    """wdm_select(centre) then decimate to dbp_osf samples/symbol (wdm_run.cpp:33-35)."""
    sel = dsp.wdm_select(field, 0, link.spacing)
    return dsp.decimate(sel, link.osf // dbp_osf)


@dataclass
class DualPolLink:
    """The dual-polarization WDM experiment of src/tasks/parameters.h:4-19 and
    src/tasks/wdm_run.cpp:79-141 (Manakov Kerr factor 8/9, 100 km spans,
    37.5 GHz spacing), with three channels: the layout WdmPPE expects
    (src/tasks/wdm_scoring.cpp:158-187)."""
    spans: int = 20
    span_m: float = 1e5
    alpha_db_km: float = 0.2
    dispersion: float = 17e-6
    gamma: float = 1.4e-3
    kappa: float = 8.0 / 9.0
    wavelength: float = 1.55e-6
    noise_figure_db: float = 4.5
    max_phase: float = 1e-3
    max_step: float = 1e3
    baud: float = 32e9
    channels: int = 3
    spacing: float = 37.5e9
    osf: int = 16
    roll_off: float = 0.01  # rrc_shaping's default (modulation.cpp:85-96)

    def fiber(self):
        return Fiber(db_to_natural(self.alpha_db_km * 1e-3), disp_to_beta2(self.dispersion, self.wavelength),
                     self.gamma, self.span_m, self.wavelength, self.kappa)

    def gain(self):
        return db_to_linear(self.alpha_db_km * self.span_m / 1e3)

    def f0(self):
        return LIGHT_SPEED / self.wavelength


def power_node(power_index: int) -> float:
    """Launch power per channel in dBm (wdm_run.cpp:22-24)."""
    return 0.5 * power_index - 6.0


def wdm_dataset(link: DualPolLink, n_symbols: int, power_dbm: float, seed: int, ctx=None, spans=None):
    """wdm_run.cpp:79-141 on the GPU for one realization: per channel 2 x
    n_symbols 16QAM symbols at power/2 per polarization, RRC shaping, WDM
    multiplexing, `spans` adaptive-step spans with ASE (one graph-captured
    span loop), then CDC, channel selection, matched filter and a 720-step
    phase-shift equalizer per channel.  Returns (tx, rx, steps): 6-row Fields
    (rows channel * 2 + polarization, the dataset layout of save_field) of
    the transmitted symbols and the received, equalized symbols."""
    spans = link.spans if spans is None else spans
    rng = np.random.default_rng(seed)
    nch = link.channels
    codes = rng.integers(0, 16, (nch, 2, n_symbols))
    sym = dsp.qam16_map(codes, Domain(2, n_symbols, 1 / link.baud, link.f0()), batch=nch, ctx=ctx)
    sym *= np.sqrt(dbm_to_watts(power_dbm) / 2)
    sig = dsp.wdm_mux(dsp.rrc_shaping(sym, link.osf, link.roll_off), link.spacing)
    fib = link.fiber()
    ssfm = SSFM(fib)
    ssfm.set_grid(SSFM.ADAPTIVE)
    ssfm.set_maximum_phase_shift(link.max_phase)
    ssfm.set_maximum_step_size(link.max_step)
    amp = Amplifier(link.gain(), db_to_linear(link.noise_figure_db), seed=seed)
    steps = span_loop([sig], fib, ssfm, spans, after=Amplifier.AMPLIFY, amplifier=amp)[0]
    cd_compensation(sig, fib, spans)
    dom = Domain(2 * nch, n_symbols, 1 / link.baud, link.f0())
    tx, rx = Field(dom, ctx=sig.ctx), Field(dom, ctx=sig.ctx)
    pse = dsp.PhaseShiftEqualizer(720)
    for ch in range(nch):
        t = sym.slice(ch, 1)
        r = dsp.rrc_sampling(dsp.wdm_select(sig, ch - nch // 2, link.spacing), link.osf, link.roll_off)
        tx.copy_modes(2 * ch, t, 0, 2)
        rx.copy_modes(2 * ch, pse.train_equalize(t, r), 0, 2)
    return tx, rx, int(steps.sum())


def centre_rows(f: Field) -> Field:
    """Rows 2-3 (the centre channel) of a 6-row dataset field."""
    out = Field(Domain(2, f.domain.samples, f.domain.time_step, f.domain.center_frequency), batch=f.batch,
                ctx=f.ctx)
    return out.copy_modes(0, f, 2, 2)


def _timed(fn, ctx, repeat=3):
    fn()
    ctx.sync()
    t0 = time.perf_counter()
    for _ in range(repeat):
        out = fn()
    ctx.sync()
    return out, (time.perf_counter() - t0) * 1e3 / repeat


def learned_dbp(link: Link, rx_train: Field, tx_train: Field, rx_test: Field, tx_test: Field, steps_per_span=2,
                taps=63, mf_taps=63, iters=300, lr=2e-3, cnn_iters=1000, cnn_lr=3e-4, cut=100, angle_steps=720,
                seed=0, cnn_triplets=None):
    """Train the learned DBP (initialised from split-step DBP) and then the
    correction CNN (on the symbols and their perturbation triplets,
    cnn.TRIPLETS unless given) on (rx_train, tx_train); score both on the
    independent (rx_test, tx_test).  The CNN trains on three quarters of the
    training realizations and is kept only if it lowers the squared error on
    the held-out quarter by at least 0.5 %; otherwise the learned DBP's output
    passes through unchanged (plain learned DBP is the fallback).  Returns a
    dict of Q per realization and GPU times."""
    from .cnn import TRIPLETS, CorrectionCNN, he_init
    cnn_triplets = TRIPLETS if cnn_triplets is None else tuple(cnn_triplets)
    from .ldbp import LearnedDBP, rrc_response
    ctx = rx_train.ctx
    B = rx_train.batch
    n2 = rx_train.domain.samples
    ns = tx_train.domain.samples
    fib = link.fiber()
    model = LearnedDBP(link.spans, steps_per_span, taps, mf_taps, n2, B, 1 / np.sqrt(link.gain()), ctx=ctx)
    model.init_from_dbp(fib.alpha, fib.beta2, fib.gamma, fib.kappa, link.span_m, rx_train.domain.time_step,
                        rrc_response(ns, n2 // ns, link.roll_off, ctx=ctx))
    pse = dsp.PhaseShiftEqualizer(angle_steps)
    # The reference equalizes the DBP output's constant phase (mostly the mean
    # cross-phase modulation of the neighbour channels) with the phase-shift
    # equalizer; fold the training set's angle into the matched filter so
    # that training starts from the equalized DBP.
    ang = pse.estimate(tx_train, model.forward(rx_train))
    model.rotate_output(float(np.angle(np.mean(np.exp(1j * ang)))))
    q_init = dsp.q2_factor(tx_test, pse.train_equalize(tx_test, model.forward(rx_test)), cut)
    t0 = time.perf_counter()
    hist = model.fit(rx_train, tx_train, iters=iters, lr=lr)
    ctx.sync()
    train_s = time.perf_counter() - t0
    y_test, ms = _timed(lambda: model.forward(rx_test), ctx)
    q_ldbp = dsp.q2_factor(tx_test, pse.train_equalize(tx_test, y_test), cut)
    y_train = model.forward(rx_train)
    p_rms = float(np.sqrt(np.mean(np.abs(tx_train.numpy(np.complex64)) ** 2)))
    nv = max(1, B // 4) if B > 1 else 0
    nt = B - nv
    y_fit, t_fit = (y_train.slice(0, nt), tx_train.slice(0, nt)) if nv else (y_train, tx_train)
    net = CorrectionCNN(ns, nt, p_rms, ctx=ctx, triplets=cnn_triplets)
    # a small random last layer (1 % of He scale): a zero one leaves only the
    # output biases with a gradient in the first step, and Adam's first
    # full-size moves then tend to switch the hidden ReLUs off for good
    net.set_params(he_init(np.random.default_rng(seed), zero_last=False, n_triplets=len(cnn_triplets),
                           last_scale=1e-2))
    t0 = time.perf_counter()
    chist = net.fit(y_fit, t_fit, iters=cnn_iters, lr=cnn_lr)
    ctx.sync()
    cnn_train_s = time.perf_counter() - t0
    params = net.get_params()[0]
    accepted, val = True, None
    if nv:
        v = CorrectionCNN(ns, nv, p_rms, ctx=ctx, triplets=cnn_triplets)
        y_val, t_val = y_train.slice(nt, nv), tx_train.slice(nt, nv)
        v.set_params(params)
        loss_val = v.loss_grad(y_val, t_val)
        v.set_params(v.identity_params(params))
        loss_id = v.loss_grad(y_val, t_val)
        accepted = loss_val < 0.995 * loss_id
        val = (loss_val, loss_id)
        if not accepted:
            params = v.identity_params(params)
    apply = CorrectionCNN(ns, rx_test.batch, p_rms, ctx=ctx, triplets=cnn_triplets)
    apply.set_params(params)
    z_test, ms_cnn = _timed(lambda: apply.forward(y_test), ctx)
    q_cnn = dsp.q2_factor(tx_test, pse.train_equalize(tx_test, z_test), cut)
    return {"q_init": q_init, "q_learned": q_ldbp, "q_learned_cnn": q_cnn, "ms_learned": ms,
            "ms_learned_cnn": ms + ms_cnn, "loss_first": hist[0], "loss_last": hist[-1],
            "cnn_loss_first": chist[0], "cnn_loss_last": chist[-1], "cnn_accepted": bool(accepted),
            "cnn_validation": val, "train_s": train_s, "cnn_train_s": cnn_train_s}


def plain_dbp_q(link: Link, rx2: Field, tx: Field, steps_per_span, cut=100, angle_steps=720):
    """backward_propagation with UNIFORM steps (systems.cpp:86-103), matched
    filter, phase-shift equalizer, Q per realization and the DBP time (timed
    like the learned DBP: one warm-up, then the mean of 3 runs)."""
    s = SSFM(link.fiber(), steps_per_span)
    f = rx2.copy()

    def run():
        f.assign(rx2)
        backward_propagation(f, link.fiber(), s, link.gain(), link.spans)
        return f

    f, ms = _timed(run, rx2.ctx)
    sym = dsp.rrc_sampling(f, rx2.domain.samples // tx.domain.samples, link.roll_off)
    eq = dsp.PhaseShiftEqualizer(angle_steps).train_equalize(tx, sym)
    return dsp.q2_factor(tx, eq, cut), ms


def learned_vs_plain(link: Link, power_dbm, n_symbols=1 << 15, batch=8, seed=0, ctx=None, steps_per_span=4,
                     plain_steps=(1, 4, 100), iters=300, lr=3e-4, cnn_iters=1000, cnn_lr=3e-4, taps=63,
                     mf_taps=255, cnn_triplets=None):
    """Learned DBP at `steps_per_span` (and with the correction CNN) against
    plain DBP on one link and launch power: independent training and test sets
    of `batch` realizations x `n_symbols` (fresh symbols and ASE), propagated
    on the GPU (ADAPTIVE steps, EDFA with ASE), the centre channel at 2
    samples/symbol.  Returns {name: {"q_db": mean Q over the test set, "ms":
    DBP time over the test set}}."""
    a, ta = wdm_transmitter(link, n_symbols, batch, power_dbm, seed=seed + 1, ctx=ctx)
    b, tb = wdm_transmitter(link, n_symbols, batch, power_dbm, seed=seed + 2, ctx=ctx)
    propagate(link, a, seed=seed + 3)
    propagate(link, b, seed=seed + 4)
    ra, rb = centre_channel(link, a), centre_channel(link, b)
    del a, b
    out = {}
    for k in plain_steps:
        q, ms = plain_dbp_q(link, rb, tb, k)
        out["plain_%d" % k] = {"q_db": float(np.mean(q)), "ms": ms}
    r = learned_dbp(link, ra, ta, rb, tb, steps_per_span=steps_per_span, taps=taps, mf_taps=mf_taps, iters=iters,
                    lr=lr, cnn_iters=cnn_iters, cnn_lr=cnn_lr, cnn_triplets=cnn_triplets)
    out["learned_%d" % steps_per_span] = {"q_db": float(np.mean(r["q_learned"])), "ms": r["ms_learned"],
                                          "train_s": r["train_s"]}
    out["learned_%d_cnn" % steps_per_span] = {"q_db": float(np.mean(r["q_learned_cnn"])),
                                              "ms": r["ms_learned_cnn"], "train_s": r["cnn_train_s"],
                                              "accepted": r["cnn_accepted"]}
    return out
