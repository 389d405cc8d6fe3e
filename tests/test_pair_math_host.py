"""The Morse pair math the kernels share (jmd::morse_terms, host/device),
compiled for the host and checked against the FP64 oracle: energy, U'/r,
U'' and the sigma / epsilon derivatives of U and U'/r, inside the onset
radius and in the switching shell (energy.py:346-440, 534-580).  CPU only;
needs nvcc (skipped without it)."""
import shutil
import subprocess
from pathlib import Path

import numpy as np
import pytest

from oracle import md_oracle as O

ROOT = Path(__file__).resolve().parent.parent


@pytest.fixture(scope='module')
def driver(tmp_path_factory):
    nvcc = shutil.which('nvcc') or '/usr/local/cuda/bin/nvcc'
    if not Path(nvcc).exists():
        pytest.skip('nvcc is not available')
    exe = tmp_path_factory.mktemp('pairmath') / 'pair_math_host'
    subprocess.run([nvcc, '-O2', '-std=c++17', '--expt-relaxed-constexpr', '-x', 'cu',
                    str(ROOT / 'tests' / 'pair_math_host.cu'), '-o', str(exe)], check=True)
    return exe


def _run(exe, rows):
    text = '\n'.join(' '.join(f'{v:.9g}' for v in row) for row in rows) + '\n'
    out = subprocess.run([str(exe)], input=text, capture_output=True, text=True, check=True)
    return np.array([[float(v) for v in l.split()] for l in out.stdout.strip().split('\n')])


def _table_row(r, sig, eps, alp, ro, rc):
    """The kernel's inputs as the pair table builds them (float32 radii, the
    switch denominator in f64 then rounded)."""
    ro2 = np.float32(np.float32(ro) * np.float32(ro))
    rc2 = np.float32(np.float32(rc) * np.float32(rc))
    den = float(rc2) - float(ro2)
    inv_den = np.float32(1.0 / den ** 3) if den > 0 else np.float32(0.0)
    return [np.float32(r) * np.float32(r), sig, eps, alp, ro2, rc2, inv_den]


@pytest.mark.parametrize('sig,eps,alp', [(1.0, 5.0, 5.0), (1.3, 0.7, 2.5), (0.8, 2.0, 9.0)])
def test_morse_terms_match_oracle(driver, sig, eps, alp):
    ro, rc = 2.0, 2.5
    r = np.concatenate([np.linspace(0.6 * sig, 1.95, 40), np.linspace(2.01, 2.49, 20)])
    got = _run(driver, [_table_row(x, sig, eps, alp, ro, rc) for x in r])
    spec = O.PairSpec(kind='morse', sigma=sig, epsilon=eps, alpha=alp, r_onset=ro, r_cutoff=rc)
    U, dU, d2U = O.pair_terms(spec, r)
    scale = max(1.0, np.abs(U).max())
    np.testing.assert_allclose(got[:, 0], U, rtol=2e-5, atol=2e-6 * scale)
    np.testing.assert_allclose(got[:, 1], dU / r, rtol=2e-5, atol=2e-5 * np.abs(dU / r).max())
    np.testing.assert_allclose(got[:, 2], d2U, rtol=2e-4, atol=2e-5 * np.abs(d2U).max())
    # parameter derivatives against central differences of the oracle
    h = 1e-6
    for col_U, col_g, key, base in ((3, 4, 'sigma', sig), (5, 6, 'epsilon', eps)):
        kw = dict(sigma=sig, epsilon=eps, alpha=alp, r_onset=ro, r_cutoff=rc)
        kw[key] = base + h
        Up, dUp, _ = O.pair_terms(O.PairSpec(kind='morse', **kw), r)
        kw[key] = base - h
        Um, dUm, _ = O.pair_terms(O.PairSpec(kind='morse', **kw), r)
        fdU, fdg = (Up - Um) / (2 * h), (dUp - dUm) / (2 * h) / r
        np.testing.assert_allclose(got[:, col_U], fdU, rtol=1e-4, atol=1e-5 * np.abs(fdU).max())
        np.testing.assert_allclose(got[:, col_g], fdg, rtol=1e-4, atol=1e-5 * np.abs(fdg).max())


def test_morse_terms_plain_and_truncated(driver):
    """With r_onset = r_cutoff (hard truncation, no switch) and with infinite
    radii (plain Morse) the switch is 1 inside the cutoff."""
    r = np.linspace(0.7, 2.4, 30)
    inf = np.float32(np.inf)
    plain = _run(driver, [[np.float32(x) ** 2, 1.0, 5.0, 5.0, inf, inf, 0.0] for x in r])
    trunc = _run(driver, [_table_row(x, 1.0, 5.0, 5.0, 2.5, 2.5) for x in r])
    U, dU, d2U = O.morse(r, 1.0, 5.0, 5.0)
    for got in (plain, trunc):
        np.testing.assert_allclose(got[:, 0], U, rtol=2e-5, atol=1e-5)
        np.testing.assert_allclose(got[:, 1], dU / r, rtol=2e-5, atol=1e-4)
        np.testing.assert_allclose(got[:, 2], d2U, rtol=2e-4, atol=1e-3)
