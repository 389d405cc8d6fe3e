"""Writes the golden fixtures in this folder from the reference's test data.

Run once where the reference checkout is present:
    python tests/golden/make_golden.py /path/to/jax-md
It reads only the reference's data files (tests/data/...), never its code, and
writes small .npz fixtures that the test suite loads on any machine:

  lammps_lj_stress.npz   LAMMPS LJ dump (108 atoms, box 5.0388) used by
                         tests/quantity_test.py:436-455: fractional positions,
                         velocities, energy per atom -4.3523016 and the stress.
  jammed_soft_sphere_2d.npz  2D bidisperse jammed packing used by
                         tests/quantity_test.py:134-150 (simulation_test_state.npy):
                         positions, species, sigma matrix, box, energy, pressure.
"""
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent


def lammps(ref: Path):
    # parser follows jax_md/test_util.py:370-420 (load_lammps_stress_data)
    lines = (ref / 'tests/data/lammps_lj_stress_test_states').read_text().split('\n')
    n = int(lines[3])
    box = float(lines[5].split(' ')[-1])
    R, V = [], []
    for l in lines[9:-1]:
        v = [float(x) for x in l.split(' ')]
        R.append(v[:3])
        V.append(v[3:])
    res = [[float(x) for x in l.split(' ') if x not in ('', ' ')]
           for l in (ref / 'tests/data/lammps_lj_stress_test').read_text().split('\n')]
    res = [r for r in res if r]
    C = res[0][2:]
    stress = np.array([[C[0], C[3], C[4]], [C[3], C[1], C[5]], [C[4], C[5], C[2]]])
    assert len(R) == n
    np.savez(HERE / 'lammps_lj_stress.npz', fractional_position=np.array(R),
             velocity=np.array(V), box=np.float64(box), energy_per_atom=np.float64(res[0][1]),
             stress=stress)


def jammed(ref: Path):
    # layout follows jax_md/test_util.py:336-367 (load_jammed_state)
    with open(ref / 'tests/data/simulation_test_state.npy', 'rb') as f:
        arrs = [np.load(f) for _ in range(7)]
    names = ['fractional_position', 'real_position', 'species', 'sigma', 'box', 'energy',
             'pressure']
    np.savez(HERE / 'jammed_soft_sphere_2d.npz', **dict(zip(names, arrs)))


if __name__ == '__main__':
    if len(sys.argv) != 2:
        sys.exit('usage: python tests/golden/make_golden.py /path/to/jax-md')
    ref = Path(sys.argv[1])
    lammps(ref)
    jammed(ref)
    print('wrote', sorted(p.name for p in HERE.glob('*.npz')))
