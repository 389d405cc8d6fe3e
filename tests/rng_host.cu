// Host driver for the generator unit test (tests/test_rng_host.py): runs the
// kernels' shared host/device Philox4x32-10 + Box-Muller code on the CPU.
// Reads lines "seed step atom" and prints the four words and four normals;
// a line "W w0 w1 w2 w3" prints the uniforms and the normals of four given
// words instead.
#include <cstdio>

#include "../jax_md_gb300/csrc/rng.cuh"

int main() {
  char tag[32];
  while (std::scanf("%31s", tag) == 1) {
    if (tag[0] == 'W') {
      jmd::Words4 w;
      if (std::scanf("%u %u %u %u", &w.w[0], &w.w[1], &w.w[2], &w.w[3]) != 4) return 1;
      float z[4];
      jmd::normals_from_words(w, z);
      std::printf("%.17g %.17g %.17g %.17g %.9g %.9g %.9g %.9g\n",
                  (double)jmd::word_to_unit(w.w[0]), (double)jmd::word_to_unit(w.w[1]),
                  (double)jmd::word_to_unit(w.w[2]), (double)jmd::word_to_unit(w.w[3]), z[0], z[1],
                  z[2], z[3]);
      continue;
    }
    unsigned long long seed, step;
    unsigned atom;
    if (std::sscanf(tag, "%llu", &seed) != 1) return 1;
    if (std::scanf("%llu %u", &step, &atom) != 2) return 1;
    const jmd::Words4 w = jmd::philox4x32_10(atom, 0u, (uint32_t)step, (uint32_t)(step >> 32),
                                             (uint32_t)seed, (uint32_t)(seed >> 32));
    float z[4];
    jmd::langevin_normals(seed, step, atom, z);
    std::printf("%u %u %u %u %.9g %.9g %.9g %.9g\n", w.w[0], w.w[1], w.w[2], w.w[3], z[0], z[1],
                z[2], z[3]);
  }
  return 0;
}
