"""The benchmark workloads have the shapes their configurations state and are
reproducible (seeded), so the bench line's ``config`` describes what ran.

single_600_o8: 600x600, dt 0.05 s, nt 3000, 8th-order FD, 300 frequencies in
0.01-0.2 Hz, two reference stations, 40 receivers, random media with 10 % std,
ring noise source.  structure_512: 512x512, nt 2500, snapshots every 5 steps,
200 frequencies, one reference station with 20 receivers around it.
batch_uneven: 32 stations on grids of 256, 384, 512 or 800 points square, nt
in 1500-4000, dt from CFL 0.5 at 4000 m/s, 4th order, taper 30 points, four
frequency bands.  plain_cpu_300: 300x300, dt 0.1 s, nt 1200, 4th order, 200
frequencies, 10 receivers, taper 20 points, +-5 % smoothed mu.
"""
import numpy as np

from fd2d_noise_gb300 import workloads


def test_single_600_o8():
    w = workloads.single_600_o8()
    c = w.cfg
    assert (c.nx, c.nz, c.dt, c.nt, c.order, c.n_sample) == (600, 600, 0.05, 3000, 8, 300)
    assert c.f_sample[0] == 0.01 and abs(c.f_sample[-1] - 0.2) < 1e-12
    assert w.ref_stations.shape == (2, 2) and w.receivers.shape == (40, 2)
    assert w.spectrum.shape == (300, 1) and w.source_dist.shape[:2] == (600, 600)
    rel = w.mu / 4.8e10 - 1
    assert abs(rel.std() - 0.10) < 1e-3 and abs(rel.mean()) < 1e-12
    assert w.gpt_per_station() == 600 * 600 * (3000 + 5999)
    # ring: zero away from the ring, positive on it
    assert (w.source_dist == 0).mean() > 0.5 and w.source_dist.max() > 0
    w2 = workloads.single_600_o8()
    for k in ("mu", "rho", "ref_stations", "receivers", "spectrum", "source_dist"):
        assert np.array_equal(getattr(w, k), getattr(w2, k)), k


def test_structure_512():
    w = workloads.structure_512()
    c = w.cfg
    assert (c.nx, c.nz, c.nt, c.fw_nth, c.freq_samp, c.n_sample) == (512, 512, 2500, 5, 5, 200)
    assert w.ref_stations.shape == (1, 2) and w.receivers.shape == (20, 2)
    r = np.hypot(*(w.receivers - w.ref_stations[0]).T)
    assert np.allclose(r, r[0])  # a ring around the reference station
    # arrivals (~4 km/s) inside the 100-200 s measurement window
    assert 100.0 < r[0] / 4000.0 < 200.0 and (c.nt - 1) * c.dt >= 200.0
    assert w.mu_true is not None and w.mu_true.shape == w.mu.shape and np.any(w.mu_true != w.mu)


def test_batch_uneven():
    b = workloads.batch_uneven()
    assert len(b.stations) == 32
    sizes = {s.cfg.nx for s in b.stations}
    assert sizes <= {256, 384, 512, 800} and len(sizes) >= 3
    for s in b.stations:
        c = s.cfg
        assert c.nx == c.nz and 1500 <= c.nt <= 4000 and c.order == 4 and c.n_basis_fct == 4
        assert abs(c.dt - 0.5 * c.dx / 4000.0) < 1e-15 and abs(c.absorb_width - 30 * c.dx) < 1e-9
        assert s.source_dist.shape == (c.nx, c.nz, 4) and np.all(s.spectrum == 1.0)
    assert b.gpt_per_step() == sum(s.cfg.npts * (s.cfg.nt + s.cfg.ntc) for s in b.stations)


def test_plain_cpu_300():
    w = workloads.plain_cpu_300()
    c = w.cfg
    assert (c.nx, c.nz, c.dt, c.nt, c.order, c.n_sample) == (300, 300, 0.1, 1200, 4, 200)
    assert w.receivers.shape == (10, 2) and w.ref_stations.shape == (1, 2)
    assert abs(c.absorb_width - 20 * c.dx) < 1e-9
    assert abs(np.abs(w.mu / 4.8e10 - 1).max() - 0.05) < 1e-12
