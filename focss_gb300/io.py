"""Dataset files of the reference, so fields produced on the GPU feed its
offline scoring tasks (and recorded datasets feed the GPU receivers).

* Transmission CSV (src/focss/functions.cpp:174-221): one line per sample,
  ``tx_0.re,tx_0.im,...,tx_M-1.re,tx_M-1.im,rx_0.re,...,rx_M-1.im``, values
  printed with 15 significant digits (``std::ofstream::precision(15)``).
* Field binary (src/tasks/wdm_run.cpp:55-77, read back by
  src/tasks/wdm_scoring.cpp:79-103): four native ints ``n_ch, n_samples,
  n_modes, flags=0`` then, sample-major, channel, mode: complex128 values.

Host-side file formats: fields are read from / written to the device with one
download / upload; no compute happens here.
"""
from __future__ import annotations

import os

import numpy as np

from .api import Field


def _modes_samples(x):
    """(modes, samples) complex128 of realization 0 of a Field, or an array."""
    if isinstance(x, Field):
        return x.numpy(np.complex128)[0]
    a = np.asarray(x, np.complex128)
    return a[None] if a.ndim == 1 else a


def _g15(v: float) -> str:
    return "%.15g" % v


def save_transmission(path, tx, rx):
    """save_transmission(filename, tx, rx) (functions.cpp:174-208)."""
    t, r = _modes_samples(tx), _modes_samples(rx)
    if t.shape != r.shape:
        raise ValueError("tx and rx must have the same modes and samples")
    modes, samples = t.shape
    cols = np.empty((samples, 4 * modes), np.float64)
    for m in range(modes):
        cols[:, 2 * m] = t[m].real
        cols[:, 2 * m + 1] = t[m].imag
        cols[:, 2 * modes + 2 * m] = r[m].real
        cols[:, 2 * modes + 2 * m + 1] = r[m].imag
    with open(path, "w") as fh:
        fh.writelines(",".join(map(_g15, row)) + "\n" for row in cols)


def load_transmission(path, modes: int, samples: int):
    """load_transmission(filename, &tx, &rx) (functions.cpp:190-221): returns
    (tx, rx) as (modes, samples) complex128 arrays."""
    data = np.loadtxt(path, delimiter=",", ndmin=2, max_rows=samples)
    if data.shape != (samples, 4 * modes):
        raise ValueError("expected %d rows of %d values, got %s" % (samples, 4 * modes, data.shape))
    tx = (data[:, 0:2 * modes:2] + 1j * data[:, 1:2 * modes:2]).T.copy()
    rx = (data[:, 2 * modes::2] + 1j * data[:, 2 * modes + 1::2]).T.copy()
    return tx, rx


def _field_path(set_dir, tag, index):
    return os.path.join(str(set_dir), str(tag), "%d.bin" % index)


def save_field(channels, set_dir, tag, index: int):
    """save_field(data, set, tag, index) (wdm_run.cpp:55-77).  `channels` is a
    list of (modes, samples) arrays / Fields, or one Field whose realizations
    are the channels."""
    if isinstance(channels, Field):
        arr = channels.numpy(np.complex128)            # (n_ch, modes, samples)
    else:
        arr = np.stack([_modes_samples(c) for c in channels])
    n_ch, n_modes, n_samples = arr.shape
    path = _field_path(set_dir, tag, index)
    with open(path, "wb") as fh:
        np.array([n_ch, n_samples, n_modes, 0], np.int32).tofile(fh)
        np.ascontiguousarray(arr.transpose(2, 0, 1)).astype(np.complex128).tofile(fh)
    return path


def load_field(set_dir, tag, index: int):
    """load_field(set, tag, index) (wdm_scoring.cpp:79-103): an
    (n_ch * n_modes, n_samples) complex128 array, envelope = ch * n_modes + mode."""
    path = _field_path(set_dir, tag, index)
    with open(path, "rb") as fh:
        n_ch, n_samples, n_modes, _flags = np.fromfile(fh, np.int32, 4)
        data = np.fromfile(fh, np.complex128, n_ch * n_modes * n_samples)
    if data.size != n_ch * n_modes * n_samples:
        raise ValueError("truncated field file %s" % path)
    return data.reshape(n_samples, n_ch * n_modes).T.copy()
