"""The reference's on-disk formats (MAT v5/v7 via scipy.io) and calculate_data.

    array_<n_ref>_ref.mat          'array', 'ref_stat'      code/calculate_data.m:222
    data_<n_ref>_ref_<nb>.mat      'c_data', 't'            code/calculate_data.m:223
    G_fft_<i>.mat                  'x'                      code/parsave.m:4 (Green-spectrum cache,
                                                            eval_objective_and_gradient.m:44-50)
    G_2_<i>.mat                    'G_2'                    README.md:51 (no shipped code writes it:
                                                            here the conjugated G_fft of station i)

``c_data`` stacks the correlations of reference station i (1-based) in rows
(i-1)*n_rec + 1 .. i*n_rec (code/calculate_data.m:206-209).  MAT v7.3 (HDF5)
would need h5py, which this environment lacks.
"""
from __future__ import annotations

import os
from typing import Optional

import numpy as np


def _savemat(path, d):
    import scipy.io
    scipy.io.savemat(path, d, do_compression=True, oned_as="row")


def _loadmat(path):
    import scipy.io
    return scipy.io.loadmat(path)


def array_path(out_dir, n_ref):
    return os.path.join(out_dir, f"array_{n_ref}_ref.mat")


def data_path(out_dir, n_ref, nb):
    return os.path.join(out_dir, f"data_{n_ref}_ref_{nb}.mat")


def save_array(out_dir, array, ref_stat) -> str:
    ref_stat = np.atleast_2d(np.asarray(ref_stat, dtype=np.float64))
    p = array_path(out_dir, ref_stat.shape[0])
    _savemat(p, {"array": np.asarray(array, dtype=np.float64), "ref_stat": ref_stat})
    return p


def load_array(path):
    d = _loadmat(path)
    return d["array"], d["ref_stat"]


def save_data(out_dir, c_data, t, n_ref, nb) -> str:
    p = data_path(out_dir, n_ref, nb)
    _savemat(p, {"c_data": np.asarray(c_data, dtype=np.float64),
                 "t": np.asarray(t, dtype=np.float64).reshape(1, -1)})
    return p


def load_data(path):
    d = _loadmat(path)
    return d["c_data"], d["t"]


def save_green(out_dir, i, G_fft, name="G_2") -> str:
    """G_2_<i>.mat ('G_2') or, with name='G_fft', the cache G_fft_<i>.mat ('x')."""
    if name == "G_2":
        p, var = os.path.join(out_dir, f"G_2_{i}.mat"), "G_2"
    else:
        p, var = os.path.join(out_dir, f"G_fft_{i}.mat"), "x"
    _savemat(p, {var: np.asarray(G_fft)})
    return p


def load_green(path):
    d = _loadmat(path)
    return d["G_2"] if "G_2" in d else d["x"]


def receivers_of(array, src):
    """array(find(~ismember(array, src, 'rows')), :)"""
    a = np.asarray(array, dtype=np.float64)
    return a[~np.all(a == np.asarray(src, dtype=np.float64).reshape(1, 2), axis=1)]


def calculate_data(mu, rho, spectrum, source_dist, array, ref_stat, *, cfg, out_dir: Optional[str] = None,
                   save_green_spectra: bool = False, precision: str = "fp32", device: int = 0):
    """The station loop of code/calculate_data.m:186-223 on the GPU: for each
    reference station the Green function and the correlation wavefield, the
    correlations stacked into c_data, and (with ``out_dir``) the array and
    data files.  Without Green-spectrum files the stations run as one batch
    (lanes of the same launches).  Returns (c_data, t)."""
    from . import _lib, solvers
    ref_stat = np.atleast_2d(np.asarray(ref_stat, dtype=np.float64))
    n_ref = ref_stat.shape[0]
    n_rec = np.asarray(array).shape[0] - 1
    t = (-(cfg.nt - 1) + np.arange(cfg.ntc)) * cfg.dt
    c_data = np.zeros((n_ref * n_rec, cfg.ntc))
    if save_green_spectra:
        for i in range(n_ref):
            src = ref_stat[i:i + 1]
            rec = receivers_of(array, src)
            G, _, _ = solvers.run_forward1_green(mu, rho, src, rec, 0, None, None, cfg=cfg, precision=precision,
                                                 device=device)
            if out_dir:
                save_green(out_dir, i + 1, G)
            c, _ = solvers.run_forward2_correlation(mu, rho, G, spectrum, source_dist, rec, 0, None, None, cfg=cfg,
                                                    precision=precision, device=device)
            c_data[i * n_rec:(i + 1) * n_rec] = np.asarray(c).reshape(-1, cfg.ntc)[:n_rec]
    else:
        import ctypes
        ctx = solvers.context(device, precision)
        cc = cfg.to_c()
        mu_ = np.asfortranarray(mu, dtype=np.float64)
        rho_ = np.asfortranarray(rho, dtype=np.float64)
        spec = np.asfortranarray(np.asarray(spectrum, dtype=np.float64).reshape(cfg.n_sample, -1))
        sd = np.asfortranarray(source_dist, dtype=np.float64)
        n_dist = 1 if sd.ndim == 2 else sd.shape[2]
        srcs, recs, outs = [], [], []
        jobs = (_lib.FD2DJob * n_ref)()
        for i in range(n_ref):
            srcs.append(np.asfortranarray(ref_stat[i:i + 1]))
            recs.append(np.asfortranarray(receivers_of(array, ref_stat[i:i + 1])))
            outs.append(np.zeros((recs[i].shape[0], cfg.ntc), order="F"))
            j = jobs[i]
            j.cfg = ctypes.pointer(cc)
            j.mu, j.rho = mu_.ctypes.data, rho_.ctypes.data
            j.spectrum, j.n_noise_sources = spec.ctypes.data, spec.shape[1]
            j.source_dist, j.n_dist = sd.ctypes.data, n_dist
            j.src, j.rec, j.nr = srcs[i].ctypes.data, recs[i].ctypes.data, recs[i].shape[0]
            j.correlations = outs[i].ctypes.data
        _lib.check(ctx.L.fd2d_correlation_batch(ctx.h, jobs, n_ref), ctx.h)
        for i in range(n_ref):
            c_data[i * n_rec:(i + 1) * n_rec] = outs[i][:n_rec]
    if out_dir:
        os.makedirs(out_dir, exist_ok=True)
        save_array(out_dir, array, ref_stat)
        save_data(out_dir, c_data, t, n_ref, cfg.n_basis_fct)
    return c_data, t
