"""Superposition and linearity of the solvers on the FP64 oracle.

- Point sources superpose: every source of code/run_forward1_green.m:152-156
  adds the same force to DS at its node, so the spectra and traces of two
  sources together are the sums of those of each alone.
- The correlation source of code/run_forward2_correlation.m:195-216 is
  real(spectrum * distribution * G_fft * coeff), linear in each of the three,
  so the correlations are linear in the noise distribution, in the spectrum
  and in the Green spectra.

These relations hold to rounding at any size; the full-size GPU test checks
linearity in the distribution on the batched FP32 form.
"""
import numpy as np

from tests.problems import media, noise_source, rel_l2, small_cfg, stations

CFG = dict(nx=36, nz=32, nt=60, order=4, K=12, fs=5, fw=1)


def test_point_sources_superpose(oracle):
    cfg = small_cfg(**CFG)
    mu, rho = media(cfg, seed=7)
    src = stations(cfg, 2, seed=8)
    rec = stations(cfg, 4, seed=9)
    G12, _, s12 = oracle.forward1_green(cfg, mu, rho, src, rec, 0)
    G1, _, s1 = oracle.forward1_green(cfg, mu, rho, src[:1], rec, 0)
    G2, _, s2 = oracle.forward1_green(cfg, mu, rho, src[1:], rec, 0)
    assert rel_l2(G12, G1 + G2) < 1e-13 and rel_l2(s12, s1 + s2) < 1e-13
    assert rel_l2(G1, G2) > 0.1  # the two sources are different problems


def test_correlations_are_linear(oracle):
    cfg = small_cfg(**CFG)
    mu, rho = media(cfg, seed=7)
    src, rec = stations(cfg, 1, seed=8), stations(cfg, 4, seed=9)
    spec, sd1 = noise_source(cfg, seed=1)
    _, sd2 = noise_source(cfg, seed=2)
    G, _, _ = oracle.forward1_green(cfg, mu, rho, src, rec, 0)
    Gb, _, _ = oracle.forward1_green(cfg, mu, rho, stations(cfg, 1, seed=10), rec, 0)

    def corr(g, sp, sd):
        return oracle.forward2_correlation(cfg, mu, rho, g, sp, sd, rec, 0)[0]

    c1, c2 = corr(G, spec, sd1), corr(G, spec, sd2)
    assert rel_l2(corr(G, spec, sd1 + 2.5 * sd2), c1 + 2.5 * c2) < 1e-12
    spec2 = np.cos(np.arange(cfg.n_sample))[:, None] * spec
    assert rel_l2(corr(G, spec - 0.5 * spec2, sd1), c1 - 0.5 * corr(G, spec2, sd1)) < 1e-12
    assert rel_l2(corr(G + 3.0 * Gb, spec, sd1), c1 + 3.0 * corr(Gb, spec, sd1)) < 1e-12
