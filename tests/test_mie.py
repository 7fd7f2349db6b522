"""The method's RCS against the Mie series of a PEC sphere.

CPU part: the oracle's dense MoM (Zmn_MoM, modMoM.f90:219-265) on the
r = 0.5 lambda icosphere (1280 triangles, 1920 RWG), x-polarised plane wave
from -z, bistatic cut theta = 0..180 deg at phi = 0 and 90 deg
(calc_E / sigmaRCS, modRCS.f90:339-432).  The GPU part (the MLFMA solve on
the r = 3 lambda sphere) lives in test_gpu_mie.py.
"""
import numpy as np

from lywell_gb300 import meshes
from oracle import core, mie
from oracle.rwg import RWG


def test_mie_series_limits():
    # Rayleigh limit 9 pi a^2 (ka)^4 and the optical limit pi a^2
    r = 0.01
    k = 2 * np.pi
    assert abs(mie.sphere_backscatter(r, 1.0) / (9 * np.pi * r * r * (k * r) ** 4) - 1) < 2e-3
    assert abs(mie.sphere_backscatter(20.0, 1.0) / (np.pi * 400.0) - 1) < 2e-3
    # backscatter from the bistatic sum at theta = pi, both planes
    for ph in (0.0, np.pi / 2):
        assert abs(mie.sphere_rcs(1.3, 1.0, np.pi, ph) / mie.sphere_backscatter(1.3, 1.0) - 1) < 1e-12


def test_dense_mom_rcs_against_mie():
    r = RWG(meshes.icosphere(3, 0.5))
    assert r.N == 1920
    o = core.OracleMLFMA(r, lam=1.0, ladomax=0.1)    # only the geometry is used
    Z = o.zmn_rows(0, r.N)
    d = np.array([0.0, 0.0, 1.0])
    p = np.array([1.0, 0.0, 0.0], dtype=complex)
    b = core.generar_onda(r, 1.0, d, p)
    current = np.linalg.solve(Z, b)
    th = np.deg2rad(np.arange(0.0, 181.0))
    for ph in (0.0, np.pi / 2):
        s = core.sigma_rcs(r, 1.0, current, p, th, np.full_like(th, ph))
        m = mie.sphere_rcs(0.5, 1.0, th, ph)
        err = np.abs(10 * np.log10(s) - 10 * np.log10(m))
        assert err.max() < 0.2, err.max()
