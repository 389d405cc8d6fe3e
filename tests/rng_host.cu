// Host driver for the generator unit test (tests/test_rng_host.py): runs the
// kernels' shared host/device Philox4x32-10 + Box-Muller code on the CPU.
// Reads lines "seed step atom" and prints the four words and four normals.
#include <cstdio>

#include "../jax_md_gb300/csrc/rng.cuh"

int main() {
  unsigned long long seed, step;
  unsigned atom;
  while (std::scanf("%llu %llu %u", &seed, &step, &atom) == 3) {
    const jmd::Words4 w = jmd::philox4x32_10(atom, 0u, (uint32_t)step, (uint32_t)(step >> 32),
                                             (uint32_t)seed, (uint32_t)(seed >> 32));
    float z[4];
    jmd::langevin_normals(seed, step, atom, z);
    std::printf("%u %u %u %u %.9g %.9g %.9g %.9g\n", w.w[0], w.w[1], w.w[2], w.w[3], z[0], z[1],
                z[2], z[3]);
  }
  return 0;
}
