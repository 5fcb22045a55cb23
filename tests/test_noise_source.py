"""The noise-source model against the reference's own make_noise_source.m.

tests/golden/noise_source_cases.npz holds the spectra and source
distributions that the unmodified input/make_noise_source.m (with
code/propagation/general_source.m and integration_limits.m) returns when run
by the MATLAB-subset interpreter (tests/golden/make_golden_noise.py): the
homogeneous, Gaussian ('small' and 'big' domain parameter sets) and ring
types, without and with frequency bands.  fd2d_noise_gb300.noise_source must
reproduce them to the last bit.
"""
import os

import numpy as np
import pytest

from fd2d_noise_gb300.config import Config
from fd2d_noise_gb300.noise_source import integration_limits, make_noise_source

GOLDEN = np.load(os.path.join(os.path.dirname(__file__), "golden", "noise_source_cases.npz"))
CASES = sorted({k.split("/")[0] for k in GOLDEN.files})


@pytest.mark.parametrize("name", CASES)
def test_make_noise_source_matches_reference(name):
    g = lambda k: GOLDEN[f"{name}/{k}"]  # noqa: E731
    L, n, nb, kind = float(g("L")), int(g("n")), int(g("nb")), str(g("type"))
    cfg = Config(Lx=L, Lz=L, nx=n, nz=n, dt=0.1, nt=100, order=4, n_basis_fct=nb, f_sample=g("f_sample"),
                 freq_samp=5, fw_nth=1, absorb_width=1.0)
    dist, spec = make_noise_source(kind, nb, cfg)
    ref_d, ref_s = g("dist"), g("spectrum")
    assert np.array_equal(dist.reshape(ref_d.shape, order="F"), ref_d)
    assert np.array_equal(spec, ref_s)


def test_bands_cover_every_frequency_once():
    for K, nb in ((25, 3), (31, 4), (300, 7), (12, 12)):
        lim = integration_limits(K, nb)
        assert lim[0, 0] == 1 and lim[-1, 1] == K
        assert np.all(lim[1:, 0] == lim[:-1, 1] + 1)
