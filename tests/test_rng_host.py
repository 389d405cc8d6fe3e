"""The Langevin generator the kernels use (Philox4x32-10 + Box-Muller,
jax_md_gb300/csrc/rng.cuh), compiled for the host and checked against the
oracle's independent NumPy restatement: identical 32-bit words, normals to
float32 rounding, and the moments of a standard normal.  CPU only; needs
nvcc (skipped without it)."""
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
    exe = tmp_path_factory.mktemp('rng') / 'rng_host'
    subprocess.run([nvcc, '-O2', '-std=c++17', '-x', 'cu', str(ROOT / 'tests' / 'rng_host.cu'),
                    '-o', str(exe)], check=True)
    return exe


@pytest.mark.parametrize('seed,step', [(0, 0), (12345, 7), (2 ** 40 + 3, 2 ** 33 + 5),
                                       (2 ** 64 - 1, 2 ** 64 - 1)])
def test_device_generator_matches_restatement(driver, seed, step):
    n = 300
    text = ''.join(f'{seed} {step} {i}\n' for i in range(n))
    out = subprocess.run([str(driver)], input=text, capture_output=True, text=True, check=True)
    got = np.array([l.split() for l in out.stdout.strip().split('\n')])
    w, z = O.langevin_normals(seed, step, n)
    np.testing.assert_array_equal(got[:, :4].astype(np.uint64), w.astype(np.uint64))
    np.testing.assert_allclose(got[:, 4:].astype(np.float64), z, rtol=2e-6, atol=2e-6)


def test_uniforms_are_exact_at_the_ends_of_the_word_range(driver):
    """Words near 0 and 0xFFFFFFFF: the device's float32 uniform equals the
    oracle's (2 (w >> 9) + 1) / 2^24 exactly and lies strictly inside (0, 1),
    so u0 near 1 (small Box-Muller radius) replays to float32 rounding of the
    normals rather than to the rounding of u."""
    edge = [0, 1, 511, 512, 0xFFFFFFFF, 0xFFFFFFFE, 0xFFFFFE00, 0xFFFFFDFF, 0xFFFFFC00,
            0x80000000, 0x7FFFFFFF, 0xFFFF0000]
    rng = np.random.default_rng(7)
    words = np.array([[a, b, c, d] for a in edge for b, c, d in rng.integers(0, 2 ** 32, (4, 3))],
                     dtype=np.uint64)
    words = np.concatenate([words, rng.integers(0xFFFFF000, 2 ** 32, (200, 4), dtype=np.uint64)])
    text = ''.join('W ' + ' '.join(str(int(x)) for x in w) + '\n' for w in words)
    out = subprocess.run([str(driver)], input=text, capture_output=True, text=True, check=True)
    got = np.array([l.split() for l in out.stdout.strip().split('\n')], dtype=np.float64)
    u = np.stack([O.word_to_unit(words[:, k]) for k in range(4)], 1)
    np.testing.assert_array_equal(got[:, :4], u)
    assert np.all(u > 0) and np.all(u < 1)
    z = O.normals_from_words(words)
    # the float32 Box-Muller: a few ulp of the radius and of the angle's sin/cos
    np.testing.assert_allclose(got[:, 4:], z, rtol=2e-6, atol=2e-6)


def test_draws_are_standard_normal_and_independent():
    """Moments over 400,000 draws (and across steps and seeds): mean 0,
    variance 1, no correlation between components, steps or seeds, within
    five standard errors."""
    n = 100000
    _, a = O.langevin_normals(3, 10, n)
    _, b = O.langevin_normals(3, 11, n)
    _, c = O.langevin_normals(4, 10, n)
    se = 1.0 / np.sqrt(n)
    for z in (a, b, c):
        assert np.all(np.abs(z.mean(0)) < 5 * se)
        assert np.all(np.abs(z.var(0) - 1.0) < 5 * np.sqrt(2.0) * se)
        r = np.corrcoef(z.T)
        assert np.all(np.abs(r[np.triu_indices(4, 1)]) < 5 * se)
    for x, y in ((a, b), (a, c)):
        assert np.all(np.abs((x * y).mean(0)) < 5 * se)
    assert np.abs(np.mean(a[:, 0] ** 4) - 3.0) < 5 * np.sqrt(96.0) * se   # kurtosis of N(0, 1)
