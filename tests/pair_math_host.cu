// Host driver for the pair-math unit test (tests/test_pair_math_host.py):
// evaluates the kernels' shared host/device Morse function on the CPU.
// Reads lines "r2 sigma eps alpha ro2 rc2 inv_den" from stdin and prints
// "U g hh dU_s dg_s dU_e dg_e" per line.
#include <cstdio>

#include "../jax_md_gb300/csrc/pair.cuh"

int main() {
  float r2, sigma, eps, alpha, ro2, rc2, inv_den;
  while (std::scanf("%f %f %f %f %f %f %f", &r2, &sigma, &eps, &alpha, &ro2, &rc2, &inv_den) == 7) {
    const jmd::MorseTerms m = jmd::morse_terms(r2, sigma, eps, alpha, ro2, rc2, inv_den);
    std::printf("%.9g %.9g %.9g %.9g %.9g %.9g %.9g\n", m.U, m.g, m.hh, m.dU_s, m.dg_s, m.dU_e,
                m.dg_e);
  }
  return 0;
}
