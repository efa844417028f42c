"""The oracle's element matrices against exact rational integrals
(tests/golden/element_kat.json, made by tests/golden/make_golden.py) and the
known answers of the unit-cube K0."""
import json
from pathlib import Path

import numpy as np
import pytest

KAT = json.loads((Path(__file__).parent / "golden" / "element_kat.json").read_text())


@pytest.mark.parametrize("case", KAT["stiffness"], ids=lambda c: f"{c['dx']}x{c['dy']}x{c['dz']}-nu{c['nu']}")
def test_k0_matches_exact(oracle, case):
    K = np.array(case["K0"])
    Ko = oracle.canonical_stiffness(case["dx"], case["dy"], case["dz"], case["nu"])
    assert np.abs(Ko - K).max() <= 2e-15 * np.abs(K).max()


def test_k0_fp32_mode_differs_by_float_rounding(oracle):
    K = np.array(KAT["stiffness"][0]["K0"])
    Kf = oracle.canonical_stiffness(1, 1, 1, 0.3, fp32=True)
    rel = np.abs(Kf - K).max() / np.abs(K).max()
    assert 0 < rel < 5e-7


def test_unit_cube_known_answers(oracle):
    K = oracle.canonical_stiffness(1, 1, 1, 0.3)
    assert K[0, 0] == pytest.approx(55 / 234, rel=1e-15)          # (lam + 4 mu)/9
    assert np.allclose(np.diag(K), K[0, 0], rtol=1e-14)
    assert np.abs(K - K.T).max() < 1e-15
    assert np.abs(K.sum(axis=1)).max() < 1e-15                     # translations
    mags = np.unique(np.round(np.abs(K[np.abs(K) > 1e-12]), 12))
    assert mags.size == 10
    ev = np.linalg.eigvalsh(K)
    assert np.sum(np.abs(ev) < 1e-12) == 6                          # rigid-body modes
    assert ev[6] == pytest.approx(0.0641025641, rel=1e-8)
    assert ev[-1] == pytest.approx(1.25, rel=1e-12)


@pytest.mark.parametrize("case", KAT["helmholtz"], ids=lambda c: f"{c['dx']}x{c['dy']}x{c['dz']}-q{c['quirk']}")
def test_helmholtz_matrices_match_exact(oracle, case):
    Ke, Me = oracle.scalar_matrices(case["dx"], case["dy"], case["dz"], case["quirk"])
    assert np.abs(Ke - np.array(case["Ke"])).max() < 1e-15 * 10
    assert np.abs(Me - np.array(case["Me"])).max() < 1e-15 * 10


def test_helmholtz_quirk_scales_mass(oracle):
    _, Me_q = oracle.scalar_matrices(1, 1, 1, True)
    _, Me_t = oracle.scalar_matrices(1, 1, 1, False)
    assert Me_q.sum() == pytest.approx(1.5 * Me_t.sum(), rel=1e-14)  # element 1.5 dz tall
