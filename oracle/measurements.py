"""FP64 numpy restatement of the reference's measurement code.

TEST INFRASTRUCTURE: only tests/ and the benchmark's CPU leg use it, as the
checker of the library's fd2d_make_adjoint_sources.

    make_adjoint_sources   tools/measurement/make_adjoint_sources.m:31-175
    log_amp_ratio          tools/measurement/log_amp_ratio.m:23-93
    waveform_difference    tools/measurement/waveform_difference.m:23-48
    cc_time_shift          tools/measurement/cc_time_shift.m:21-61
    amp_diff               tools/measurement/amp_diff.m:22-66
    cross_correlation_td   tools/measurement/addons/cross_correlation_td.m:7-17
    get_window             tools/measurement/addons/get_window.m:1-35

MATLAB's hann, trapz and xcorr are restated from their documented
definitions (symmetric Hann window; trapezoidal rule with unit spacing;
xcorr(x, y)(m) = sum_n x(n + m) y(n) for lags m = -(N-1) .. N-1, a direct sum
in ascending n).  Pinned against
tests/golden/measurement_cases.npz (the reference's .m files run by the
MATLAB-subset interpreter).
"""
from __future__ import annotations

import numpy as np

EPS = np.finfo(np.float64).eps


def hann(n: int) -> np.ndarray:
    if n == 1:
        return np.ones(1)
    k = np.arange(n, dtype=np.float64)
    return 0.5 * (1.0 - np.cos(2.0 * np.pi * k / (n - 1)))


def trapz(y: np.ndarray) -> float:
    acc = 0.0
    for i in range(y.size - 1):
        acc = acc + (y[i] + y[i + 1]) / 2.0
    return acc


def get_window(t, t_min, t_max, kind):
    t = np.asarray(t, dtype=np.float64).ravel()
    if t_min > t_max:
        t_min, t_max = t_max, t_min
    win = np.ones(t.size) * (t > t_min) * (t < t_max)
    if kind == "hann":
        nz = np.nonzero(win)[0]
        i1, i2 = nz[0], nz[-1]
        win[i1:i2 + 1] = hann(i2 - i1 + 1)
    elif kind == "cos_taper":
        width = abs(t_max - t_min) * 0.1
        win = win + (0.5 + 0.5 * np.cos(np.pi * (t_max - t) / width)) * (t >= t_max) * (t < t_max + width)
        win = win + (0.5 + 0.5 * np.cos(np.pi * (t_min - t) / width)) * (t > t_min - width) * (t <= t_min)
    return win


def log_amp_ratio(u, u_0, du, win_caus, t, deriv_order):
    dt = abs(t[1] - t[0])
    index = int(np.argmax(win_caus))
    if t[index] < 0:
        win_acaus = win_caus
        win_caus = win_acaus[::-1]
    else:
        win_acaus = win_caus[::-1]
    e_caus = trapz((win_caus * u) ** 2) * dt
    e_acaus = trapz((win_acaus * u) ** 2) * dt + EPS
    e0_caus = trapz((win_caus * u_0) ** 2) * dt
    e0_acaus = trapz((win_acaus * u_0) ** 2) * dt + EPS
    with np.errstate(divide="ignore"):
        A = np.log(e_caus / e_acaus)
        A0 = np.log(e0_caus / e0_acaus)
    if deriv_order == "1st":
        misfit = 0.5 * (A - A0) ** 2
        de_caus = 2 * win_caus ** 2 * u * dt
        de_acaus = 2 * win_acaus ** 2 * u * dt
        if np.sum(u_0 == 0) == t.size:
            adstf = de_caus / e_caus - de_acaus / e_acaus
        else:
            adstf = (A - A0) * (de_caus / e_caus - de_acaus / e_acaus)
    else:
        misfit = None
        de_caus = trapz(2 * win_caus ** 2 * u * du) * dt
        de_acaus = trapz(2 * win_acaus ** 2 * u * du) * dt
        adstf = ((A - A0) * (2 / e_caus * win_caus ** 2 - 2 / e_acaus * win_acaus ** 2) * du * dt
                 + (A - A0) * (-2 / e_caus ** 2 * win_caus ** 2 * u * de_caus
                               + 2 / e_acaus ** 2 * win_acaus ** 2 * u * de_acaus) * dt
                 + (2 / e_caus * win_caus ** 2 * u - 2 / e_acaus * win_acaus ** 2 * u)
                 * (de_caus / e_caus - de_acaus / e_acaus) * dt)
    return misfit, adstf[::-1]


def waveform_difference(u, u_0, du, win, t, deriv_order):
    dt = abs(t[1] - t[0])
    if deriv_order == "1st":
        misfit = 0.5 * np.sum(win ** 2 * (u - u_0) ** 2) * dt
        adstf = win ** 2 * (u - u_0) * dt
    else:
        misfit = None
        adstf = win ** 2 * du * dt
    return misfit, adstf[::-1]


def xcorr(x, y):
    """xcorr(x, y) of two real vectors of length N: lags -(N-1) .. N-1."""
    x = np.asarray(x, dtype=np.float64).ravel()
    y = np.asarray(y, dtype=np.float64).ravel()
    n = x.size
    out = np.zeros(2 * n - 1)
    for m in range(-(n - 1), n):
        acc = 0.0
        for j in range(max(0, -m), min(n, n - m)):
            acc = acc + x[j + m] * y[j]
        out[m + n - 1] = acc
    return out


def cross_correlation_td(f, g, t):
    from fd2d_noise_gb300.config import matlab_colon
    n = np.asarray(f).size
    dt = t[1] - t[0]
    t_cc = matlab_colon(-(n - 1) * dt, dt, (n - 1) * dt)
    return xcorr(g, f), t_cc


def cc_time_shift(u, u_0, win, t):
    if np.sum(u_0 == 0) == t.size:
        T = 1.0
    else:
        cc, t_cc = cross_correlation_td(win * u, win * u_0, t)
        T = t_cc[int(np.argmax(cc))]
        if abs(T) > 3.5:
            T = 0.0
    misfit = T ** 2 / 2.0
    dt = abs(t[1] - t[0])
    nt = t.size
    v = np.zeros(nt)
    v[:nt - 1] = np.diff(u) / dt
    adstf = T * (win ** 2 * v) / (np.sum((win * v) ** 2) * dt)
    return misfit, adstf[::-1]


def amp_diff(u, u_0, du, win, t, deriv_order):
    dt = abs(t[1] - t[0])
    energy_0 = np.sum((win * u_0) ** 2) * dt
    measurement = (np.sum((win * u) ** 2) * dt - energy_0) / (energy_0 + EPS)
    if deriv_order == "1st":
        if np.sum(u_0 == 0) == t.size:
            misfit = 1.0
            adstf = 2 * u[::-1] / (np.sum(u ** 2) * dt)
        else:
            misfit = measurement ** 2 / 2
            adstf = 2 * measurement * win ** 2 * u / np.sum((win * u_0) ** 2)
    else:
        misfit = None
        adstf = (2 * measurement * win ** 2 * du / energy_0 * dt
                 + 4 * win ** 2 * u / energy_0 ** 2 * np.sum(win ** 2 * u * du) * dt ** 2)
    return misfit, adstf[::-1]


def make_adjoint_sources(u, u_0, du, t, veldis, measurement, deriv_order):
    """[misfit_n, adstf] for n_rec-by-nt traces u, u_0, du."""
    t = np.asarray(t, dtype=np.float64).ravel()
    u = np.array(u, dtype=np.float64, ndmin=2)
    u_0 = np.array(u_0, dtype=np.float64, ndmin=2)
    du = np.array(du, dtype=np.float64, ndmin=2)
    nt = t.size
    dt = abs(t[1] - t[0])
    n_rec = u.shape[0]
    if veldis == "vel":
        v = np.zeros((n_rec, nt))
        v0 = np.zeros((n_rec, nt))
        v[:, :nt - 1] = np.diff(u, axis=1) / dt
        v0[:, :nt - 1] = np.diff(u_0, axis=1) / dt
        u, u_0 = v, v0
    misfit_n = np.zeros(n_rec)
    adstf = np.zeros((n_rec, nt))
    for n in range(n_rec):
        if measurement == "waveform_difference":
            left, right = t[0], t[-1]
        else:
            left, right = 100.0, 200.0
            if left < 0:
                left = t[np.nonzero(t == 0)[0][0] + 1]
            if right > t[-1]:
                right = t[-1]
            if left > t[-1]:
                raise ValueError("time series too short?")
        win = get_window(t, left, right, "cos_taper")
        if measurement == "waveform_difference":
            m, a = waveform_difference(u[n], u_0[n], du[n], win, t, deriv_order)
        elif measurement in ("cc_time_shift", "amplitude_difference"):
            if measurement == "cc_time_shift" and deriv_order != "1st":
                raise ValueError("no Hessian vector products for traveltime measurements")
            # the causal window, then [left, right] = swap(-left, -right)
            win_a = get_window(t, -right, -left, "cos_taper")
            if measurement == "cc_time_shift":
                mc, ac = cc_time_shift(u[n], u_0[n], win, t)
                ma, aa = cc_time_shift(u[n], u_0[n], win_a, t)
            else:
                mc, ac = amp_diff(u[n], u_0[n], du[n], win, t, deriv_order)
                ma, aa = amp_diff(u[n], u_0[n], du[n], win_a, t, deriv_order)
            m = mc + ma if deriv_order == "1st" else None
            a = ac + aa
        elif measurement == "log_amplitude_ratio":
            win = get_window(t, left, right, "hann")
            m, a = log_amp_ratio(u[n], u_0[n], du[n], win, t, deriv_order)
        else:
            raise ValueError(measurement)
        if deriv_order == "1st":
            misfit_n[n] = m
        adstf[n] = a
        if veldis == "vel":
            adstf[n, :nt - 1] = -np.diff(adstf[n]) / dt
    return misfit_n, adstf
