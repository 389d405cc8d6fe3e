/*
 * CPU restatement (float32, OpenMP) of the plain LJ neighbour-list MD step,
 * used as the timed CPU baseline.  TEST / BASELINE INFRASTRUCTURE ONLY: the
 * product never links or calls this file.
 *
 * Algorithm (JAX MD's, restated):
 *   cell list binning        jax_md/partition.py:421-460 (cells of side L/floor(L/c))
 *   Dense neighbour list     jax_md/partition.py:911-977 (27 cells, d^2 < c^2, no self)
 *   skin-triggered rebuild   jax_md/partition.py:1146-1154
 *   LJ x smooth cutoff       jax_md/energy.py:246-272, 534-580
 *   velocity Verlet          jax_md/simulate.py:227-243
 *   Nose-Hoover NVT          jax_md/simulate.py:444-517, 649-667 (chain in f64)
 * Forces use the full list (each atom sums its own row), as the GPU kernel.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

typedef struct {
  int n, cap, cps, ncell;
  float L, cs, cut2, rc2, ro2, inv_den, thr2;
  int *head, *next, *idx, *cnt;
  float *ref;
} md_t;

static inline float mimg(float d, float L) {
  if (d > 0.5f * L) d -= L;
  else if (d < -0.5f * L) d += L;
  return d;
}

static int cell_of(const float* x, const md_t* m) {
  int c[3];
  for (int d = 0; d < 3; ++d) {
    int q = (int)(x[d] / m->cs);
    q %= m->cps;
    if (q < 0) q += m->cps;
    c[d] = q;
  }
  return c[0] + m->cps * (c[1] + m->cps * c[2]);
}

static int build(md_t* m, const float* x) {
  int n = m->n, overflow = 0;
  for (int c = 0; c < m->ncell; ++c) m->head[c] = -1;
  for (int i = n - 1; i >= 0; --i) {  /* ascending id order per cell */
    int c = cell_of(x + 3 * i, m);
    m->next[i] = m->head[c];
    m->head[c] = i;
  }
#pragma omp parallel for schedule(static) reduction(| : overflow)
  for (int i = 0; i < n; ++i) {
    int ci = cell_of(x + 3 * i, m);
    int cx = ci % m->cps, cy = (ci / m->cps) % m->cps, cz = ci / (m->cps * m->cps);
    int k = 0;
    for (int a = -1; a <= 1; ++a)
      for (int b = -1; b <= 1; ++b)
        for (int e = -1; e <= 1; ++e) {
          int qx = (cx + a + m->cps) % m->cps, qy = (cy + b + m->cps) % m->cps,
              qz = (cz + e + m->cps) % m->cps;
          for (int j = m->head[qx + m->cps * (qy + m->cps * qz)]; j >= 0; j = m->next[j]) {
            if (j == i) continue;
            float dx = mimg(x[3 * i] - x[3 * j], m->L), dy = mimg(x[3 * i + 1] - x[3 * j + 1], m->L),
                  dz = mimg(x[3 * i + 2] - x[3 * j + 2], m->L);
            if (dx * dx + dy * dy + dz * dz < m->cut2) {
              if (k < m->cap) m->idx[(size_t)i * m->cap + k] = j;
              ++k;
            }
          }
        }
    m->cnt[i] = k;
    if (k > m->cap) overflow = 1;
  }
  memcpy(m->ref, x, sizeof(float) * 3 * (size_t)n);
  return overflow;
}

static void forces(const md_t* m, const float* x, float* f) {
#pragma omp parallel for schedule(static)
  for (int i = 0; i < m->n; ++i) {
    float fx = 0, fy = 0, fz = 0;
    int k = m->cnt[i] < m->cap ? m->cnt[i] : m->cap;
    for (int q = 0; q < k; ++q) {
      int j = m->idx[(size_t)i * m->cap + q];
      float dx = mimg(x[3 * i] - x[3 * j], m->L), dy = mimg(x[3 * i + 1] - x[3 * j + 1], m->L),
            dz = mimg(x[3 * i + 2] - x[3 * j + 2], m->L);
      float r2 = dx * dx + dy * dy + dz * dz;
      if (r2 >= m->rc2 || r2 == 0.f) continue;
      float ir2 = 1.f / r2, s6 = ir2 * ir2 * ir2, s12 = s6 * s6;
      float u = 4.f * (s12 - s6), g = 4.f * (6.f * s6 - 12.f * s12) * ir2;
      if (r2 > m->ro2) {
        float a = m->rc2 - r2, b = m->rc2 + 2.f * r2 - 3.f * m->ro2;
        float S = a * a * b * m->inv_den, dS = 12.f * a * (m->ro2 - r2) * m->inv_den;
        g = g * S + u * dS;
      }
      fx -= g * dx;
      fy -= g * dy;
      fz -= g * dz;
    }
    f[3 * i] = fx;
    f[3 * i + 1] = fy;
    f[3 * i + 2] = fz;
  }
}

static int md_setup(md_t* m, int n, float L, float r_onset, float r_cut, float skin, int cap) {
  memset(m, 0, sizeof(*m));
  m->n = n;
  m->cap = cap;
  m->L = L;
  float c = r_cut + skin;
  m->cps = (int)floorf(L / c);
  if (m->cps < 3) return -2;
  m->cs = L / (float)m->cps;
  m->ncell = m->cps * m->cps * m->cps;
  m->cut2 = c * c;
  m->rc2 = r_cut * r_cut;
  m->ro2 = r_onset * r_onset;
  double den = (double)m->rc2 - m->ro2;
  m->inv_den = (float)(1.0 / (den * den * den));
  m->thr2 = (skin * 0.5f) * (skin * 0.5f);
  m->head = malloc(sizeof(int) * m->ncell);
  m->next = malloc(sizeof(int) * n);
  m->idx = malloc(sizeof(int) * (size_t)n * cap);
  m->cnt = malloc(sizeof(int) * n);
  m->ref = malloc(sizeof(float) * 3 * (size_t)n);
  return 0;
}

static void md_free(md_t* m) {
  free(m->head);
  free(m->next);
  free(m->idx);
  free(m->cnt);
  free(m->ref);
}

/* One velocity-Verlet step (skin test, rebuild, kick, drift, forces, kick). */
static void verlet_step(md_t* m, float* x, float* p, float* f, float dt, int* rebuilds, int* bad) {
  const int n = m->n;
  const float L = m->L, h = 0.5f * dt;
  int need = 0;
#pragma omp parallel for schedule(static) reduction(| : need)
  for (int i = 0; i < n; ++i) {
    float dx = mimg(x[3 * i] - m->ref[3 * i], L), dy = mimg(x[3 * i + 1] - m->ref[3 * i + 1], L),
          dz = mimg(x[3 * i + 2] - m->ref[3 * i + 2], L);
    if (dx * dx + dy * dy + dz * dz > m->thr2) need = 1;
  }
  if (need) {
    *bad |= build(m, x);
    ++*rebuilds;
  }
#pragma omp parallel for schedule(static)
  for (int i = 0; i < 3 * n; ++i) {
    p[i] += h * f[i];
    float y = x[i] + dt * p[i];
    if (y >= L) y -= L;
    else if (y < 0.f) y += L;
    x[i] = y;
  }
  forces(m, x, f);
#pragma omp parallel for schedule(static)
  for (int i = 0; i < 3 * n; ++i) p[i] += h * f[i];
}

/* Runs `steps` NVE steps in place (x, p float32 [n*3]); returns the number of
 * rebuilds, or -1 on neighbour-list overflow.  threads <= 0: OpenMP default. */
int md_cpu_run(float* x, float* p, int n, float L, float r_onset, float r_cut, float skin,
               float dt, int cap, int steps, int threads) {
#ifdef _OPENMP
  if (threads > 0) omp_set_num_threads(threads);
#endif
  md_t m;
  if (md_setup(&m, n, L, r_onset, r_cut, skin, cap)) return -2;
  float* f = malloc(sizeof(float) * 3 * (size_t)n);
  int rebuilds = 0, bad = 0;
  bad |= build(&m, x);
  forces(&m, x, f);
  for (int s = 0; s < steps && !bad; ++s) verlet_step(&m, x, p, f, dt, &rebuilds, &bad);
  md_free(&m);
  free(f);
  return bad ? -1 : rebuilds;
}

/* One Suzuki-Yoshida substep of the Nose-Hoover chain (simulate.py:444-490),
 * f64; scales KE and multiplies *scale by the momentum factor. */
static void nhc_substep(double delta, double* xi, double* pc, const double* Q, double* KE,
                        double* scale, int M1, double dof, double kT) {
  const int M = M1 - 1;
  const double d2 = delta / 2, d4 = delta / 4, d8 = delta / 8;
  double G = pc[M - 1] * pc[M - 1] / Q[M - 1] - kT;
  pc[M] += d4 * G;
  double pnew = pc[M];
  for (int m = M - 1; m > 0; --m) {
    G = pc[m - 1] * pc[m - 1] / Q[m - 1] - kT;
    const double s = exp(-d8 * pnew / Q[m + 1]);
    pnew = s * (s * pc[m] + d4 * G);
    pc[m] = pnew;
  }
  G = 2 * *KE - dof * kT;
  double s = exp(-d8 * pc[1] / Q[1]);
  pc[0] = s * (s * pc[0] + d4 * G);
  s = exp(-d2 * pc[0] / Q[0]);
  *KE *= s * s;
  *scale *= s;
  for (int m = 0; m <= M; ++m) xi[m] += d2 * pc[m] / Q[m];
  G = 2 * *KE - dof * kT;
  for (int m = 0; m < M; ++m) {
    const double sc = exp(-d8 * pc[m + 1] / Q[m + 1]);
    pc[m] = sc * (sc * pc[m] + d4 * G);
    G = pc[m] * pc[m] / Q[m] - kT;
  }
  pc[M] += d4 * G;
}

/* Half step of the chain (simulate.py:492-507), Suzuki-Yoshida weights of
 * Yoshida 1990 (the values simulate.py:328-347 uses); returns the momentum
 * scale. */
static double nhc_half(double* xi, double* pc, const double* Q, double* KE, int M1,
                       int chain_steps, int sy_steps, double dt, double dof, double kT) {
  static const double w3[3] = {0.828981543588751, -0.657963087177502, 0.828981543588751};
  static const double w5[5] = {0.2967324292201065, 0.2967324292201065, -0.186929716880426,
                               0.2967324292201065, 0.2967324292201065};
  static const double w7[7] = {0.784513610477560, 0.235573213359357, -1.17767998417887,
                               1.31518632068391, -1.17767998417887, 0.235573213359357,
                               0.784513610477560};
  double scale = 1.0;
  if (chain_steps == 1 && sy_steps == 1) {
    nhc_substep(dt, xi, pc, Q, KE, &scale, M1, dof, kT);
    return scale;
  }
  const double* w = sy_steps == 3 ? w3 : sy_steps == 5 ? w5 : sy_steps == 7 ? w7 : NULL;
  const double delta = dt / chain_steps;
  for (int k = 0; k < chain_steps * sy_steps; ++k)
    nhc_substep(delta * (w ? w[k % sy_steps] : 1.0), xi, pc, Q, KE, &scale, M1, dof, kT);
  return scale;
}

static double kinetic(const float* p, int n) {
  double ke = 0.0;
#pragma omp parallel for schedule(static) reduction(+ : ke)
  for (int i = 0; i < 3 * n; ++i) ke += (double)p[i] * p[i];
  return 0.5 * ke;
}

static void scale_p(float* p, int n, double s) {
  const float sf = (float)s;
#pragma omp parallel for schedule(static)
  for (int i = 0; i < 3 * n; ++i) p[i] *= sf;
}

/* Runs `steps` Nose-Hoover NVT steps in place (simulate.py:649-667, unit
 * mass): chain half step with update_mass on the stored kinetic energy ->
 * momentum scale -> velocity Verlet -> kinetic energy -> chain half step ->
 * momentum scale.  The chain starts as simulate.py:436-442 builds it (zero
 * positions and momenta, masses kT tau^2, the first times 3 n); chain_out
 * [3 chain_length + 1] receives xi, p_xi, Q and the stored kinetic energy.
 * Returns the number of rebuilds, or -1 on overflow (-3: bad chain). */
int md_cpu_run_nvt(float* x, float* p, int n, float L, float r_onset, float r_cut, float skin,
                   float dt, int cap, int steps, int threads, double kT, double tau,
                   int chain_length, int chain_steps, int sy_steps, double* chain_out) {
#ifdef _OPENMP
  if (threads > 0) omp_set_num_threads(threads);
#endif
  if (chain_length < 2 || chain_length > 16 || chain_steps < 1) return -3;
  md_t m;
  if (md_setup(&m, n, L, r_onset, r_cut, skin, cap)) return -2;
  float* f = malloc(sizeof(float) * 3 * (size_t)n);
  double xi[16] = {0}, pc[16] = {0}, Q[16];
  const double dof = 3.0 * n;
  double KE = kinetic(p, n);
  int rebuilds = 0, bad = 0;
  bad |= build(&m, x);
  forces(&m, x, f);
  for (int s = 0; s < steps && !bad; ++s) {
    for (int k = 0; k < chain_length; ++k) Q[k] = kT * tau * tau;
    Q[0] *= dof;
    scale_p(p, n, nhc_half(xi, pc, Q, &KE, chain_length, chain_steps, sy_steps, dt, dof, kT));
    verlet_step(&m, x, p, f, dt, &rebuilds, &bad);
    KE = kinetic(p, n);
    scale_p(p, n, nhc_half(xi, pc, Q, &KE, chain_length, chain_steps, sy_steps, dt, dof, kT));
  }
  if (chain_out) {
    for (int k = 0; k < chain_length; ++k) {
      chain_out[k] = xi[k];
      chain_out[chain_length + k] = pc[k];
      chain_out[2 * chain_length + k] = Q[k];
    }
    chain_out[3 * chain_length] = KE;
  }
  md_free(&m);
  free(f);
  return bad ? -1 : rebuilds;
}

int md_cpu_max_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}
