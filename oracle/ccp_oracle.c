/*
 * CPU oracle of the ccp chromatin Brownian-dynamics loop — TEST
 * INFRASTRUCTURE ONLY. It is the checker of the GPU engine: only tests/,
 * __graft_entry__.smoke() and bench.py's CPU-baseline / reference legs load
 * it. Nothing in the product (tfm_gb300/) links or calls it.
 *
 * It restates, function by function, the arithmetic of the reference
 * (Marco-Mendivil-Carboni/TFM, Program/src); the reference's force code is
 * __device__-only, so there is no CPU path in the reference to link against:
 *   bonded + bending        chrsim.cu:13-76     (calc_bf)
 *   wall vector + force     chrsim.cu:79-170    (calc_wpf, calc_cf<DST|ICG>)
 *   pair forces             chrsim.cu:174-198   (calc_ppf<DST|ICG>)
 *   lamina binding          chrsim.cu:202-220   (calc_lpf), A-only: :260-273
 *   pair exclusion |i-j|<=1 chrsim.cu:250
 *   noise truncation        chrsim.cu:348-356   (|z| <= 5 on the triple)
 *   stochastic Heun         chrsim.cu:365-416, Report/Chapters/Methodology.tex:29-42
 *   cell keys               sugrid.cu:15-35
 *   overlap count           chrsim.cu:805-820
 *   contact map             chrana.cu:48-84     (calc_cm)
 *   d(s), P(s)              chrana.cu:13-45     (calc_sd_cp)
 *   Rg^2, radial density    chrana.cu:372-480   (calc_observables)
 *   confined random walk    chrsim.cu:678-802   (perform_random_walk)
 * The noise generator is the published Philox4x32-10 (Salmon et al., SC'11)
 * with Box-Muller, keyed exactly like the engine (the reference seeds cuRAND
 * with time(nullptr), so its noise is not reproducible and is not pinned).
 *
 * Forces are computed in FP64 (REAL = double) and, for trajectory drift
 * bounds and the timed CPU baseline, in an FP32 mirror (REAL = float).
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

/* bead flags (same meaning as the engine's, defined independently) */
#define F_A 1u     /* type A (LADh) */
#define F_LAD 2u   /* binds lamina-binding sites */
#define F_HEAD 4u  /* first bead of a chain */

/* force-field vector layout (double ff[FF_N]) */
enum {
  FF_POT, FF_BEND_ALL, FF_KE, FF_L0, FF_KB, FF_EATT, FF_EREP, FF_RCREP, FF_RCATT,
  FF_EW, FF_RCW, FF_EL, FF_LCO, FF_LBSDEPTH, FF_KICG, FF_RCICG, FF_DT, FF_SD, FF_MAXSTEP, FF_N
};
/* geometry vector layout (double geo[GEO_N]) */
enum { G_RN, G_RO, G_RB, G_CSL, G_N };

#define POT_WF 0
#define MODE_DST 0
#define MODE_ICG 1

/* ------------------------------------------------------------ Philox */

static void philox10(const uint32_t c_in[4], uint32_t k0, uint32_t k1, uint32_t out[4]) {
  uint32_t c0 = c_in[0], c1 = c_in[1], c2 = c_in[2], c3 = c_in[3];
  for (int r = 0; r < 10; ++r) {
    uint64_t p0 = (uint64_t)0xD2511F53u * c0;
    uint64_t p1 = (uint64_t)0xCD9E8D57u * c2;
    uint32_t n0 = (uint32_t)(p1 >> 32) ^ c1 ^ k0;
    uint32_t n1 = (uint32_t)p1;
    uint32_t n2 = (uint32_t)(p0 >> 32) ^ c3 ^ k1;
    uint32_t n3 = (uint32_t)p0;
    c0 = n0; c1 = n1; c2 = n2; c3 = n3;
    k0 += 0x9E3779B9u;
    k1 += 0xBB67AE85u;
  }
  out[0] = c0; out[1] = c1; out[2] = c2; out[3] = c3;
}

void orc_philox(const uint32_t *ctr, const uint32_t *key, uint32_t *out) {
  philox10(ctr, key[0], key[1], out);
}

/* Truncated standard normals of one bead and step, in double: counter
 * (bead, attempt, step lo, step hi), key = seed; u1 = ((x>>8)+1)/2^24,
 * u2 = (y>>8)/2^24; z = sqrt(-2 ln u1) (cos, sin)(2 pi u2). */
void orc_noise(uint32_t bead, uint64_t step, uint32_t k0, uint32_t k1, double *z) {
  for (uint32_t a = 0; a < 64; ++a) {
    uint32_t c[4] = {bead, a, (uint32_t)step, (uint32_t)(step >> 32)}, o[4];
    philox10(c, k0, k1, o);
    double u1 = (double)((o[0] >> 8) + 1u) / 16777216.0;
    double u2 = (double)(o[1] >> 8) / 16777216.0;
    double u3 = (double)((o[2] >> 8) + 1u) / 16777216.0;
    double u4 = (double)(o[3] >> 8) / 16777216.0;
    double r0 = sqrt(-2.0 * log(u1)), r1 = sqrt(-2.0 * log(u3));
    z[0] = r0 * cos(2.0 * M_PI * u2);
    z[1] = r0 * sin(2.0 * M_PI * u2);
    z[2] = r1 * cos(2.0 * M_PI * u4);
    if (fabs(z[0]) <= 5.0 && fabs(z[1]) <= 5.0 && fabs(z[2]) <= 5.0) return;
  }
  z[0] = z[1] = z[2] = 0.0;
}

/* ------------------------------------------------------------ contact predicate */

/* |a - b| < cut with d^2 = fma(dz, dz, fma(dx, dx, dy*dy)) in float and a
 * correctly rounded square root: the rounding of the reference's compiled
 * length(r[x] - r[y]) < aco in calc_cm (chrana.cu:72-73), established against
 * its output on pairs within 4 ulps of the cutoff (tests/golden/ccp_cutoff.npz). */
static int in_contact(const float *a, const float *b, float cut) {
  volatile float dx = a[0] - b[0], dy = a[1] - b[1], dz = a[2] - b[2];
  float d2 = fmaf(dz, dz, fmaf(dx, dx, dy * dy));
  return sqrtf(d2) < cut;
}

/* ------------------------------------------------------------ REAL variants */

#define ORC_ACCURATE 0
#define REAL double
#define SFX(n) n##_f64
#define RSQRT(x) (1.0 / sqrt(x))
#define SQRT sqrt
#include "oracle_impl.h"
#undef REAL
#undef SFX
#undef RSQRT
#undef SQRT
#undef ORC_ACCURATE

#define ORC_ACCURATE 1
#define REAL float
#define SFX(n) n##_f32
#define RSQRT(x) (1.0f / sqrtf(x))
#define SQRT sqrtf
#include "oracle_impl.h"
#undef REAL
#undef SFX
#undef RSQRT
#undef SQRT

/* ------------------------------------------------------------ observables */

/* Contact map and separation counts of one system by brute force over all
 * pairs i < j (calc_cm, chrana.cu:48-84; the cp of calc_sd_cp, chrana.cu:13-45).
 * map: packed lower triangle of nbins bins, pairs within one copy only, a pair
 * in one bin adds 2 (both orders), self pairs are not added.
 * ps: for each chain c (heads[c] .. heads[c+1]) counts of pairs at separation
 * s <= L/2, stored at ps[ps_off[c] + s]. */
void orc_contacts(int n, const float *xyz, float cut, int nbins, int map_len, int copy_len,
                  int n_copies, int32_t *map, int n_chains, const int32_t *heads,
                  const int32_t *ps_off, int32_t *ps) {
  int32_t *chain = (int32_t *)malloc(sizeof(int32_t) * (size_t)n);
  for (int c = 0; c < n_chains; ++c) {
    int e = (c + 1 < n_chains) ? heads[c + 1] : n;
    for (int i = heads[c]; i < e; ++i) chain[i] = c;
  }
  for (int i = 0; i < n; ++i) {
    int ci = i / copy_len, li = i - ci * copy_len;
    int mi = map && ci < n_copies && li < map_len;
    int bi = mi ? (int)(((long long)li * nbins) / map_len) : 0;
    for (int j = i + 1; j < n; ++j) {
      if (!in_contact(xyz + 3 * i, xyz + 3 * j, cut)) continue;
      if (mi) {
        int cj = j / copy_len, lj = j - cj * copy_len;
        if (cj == ci && lj < map_len) {
          int bj = (int)(((long long)lj * nbins) / map_len);
          int bx = bi > bj ? bi : bj, by = bi > bj ? bj : bi;
          map[(long long)bx * (bx + 1) / 2 + by] += (bx == by) ? 2 : 1;
        }
      }
      if (ps && chain[i] == chain[j]) {
        int c = chain[i];
        int L = ((c + 1 < n_chains) ? heads[c + 1] : n) - heads[c];
        if (j - i <= L / 2) ps[ps_off[c] + (j - i)] += 1;
      }
    }
  }
  free(chain);
}

/* Non-bonded overlaps |i - j| >= 2 closer than mis (chrsim.cu:805-820). */
long long orc_overlaps(int n, const float *xyz, float mis) {
  long long po = 0;
  for (int i = 0; i < n; ++i)
    for (int j = 0; j + 1 < i; ++j)
      if (in_contact(xyz + 3 * i, xyz + 3 * j, mis)) ++po;
  return po;
}

/* FP64 observables of one system: out[0..2] = sum r, out[3] = sum |r|^2,
 * out[4 + t*64 + b] = bead volume in radial shell b (t = A, B, all), with
 * shells r_b = R_n ((b+1)/64)^(1/3) and bead radius a (chrana.cu:372-480). */
void orc_observables(int n, const float *xyz, const uint32_t *flags, double R_n, double a,
                     double *out) {
  const int nb = 64;
  double rb[64];
  memset(out, 0, sizeof(double) * (4 + 3 * 64));
  for (int b = 0; b < nb; ++b) rb[b] = R_n * pow((b + 1.0) / nb, 1.0 / 3);
  const double vfull = (4.0 / 3.0) * M_PI * a * a * a;
  for (int i = 0; i < n; ++i) {
    double x = xyz[3 * i], y = xyz[3 * i + 1], z = xyz[3 * i + 2];
    out[0] += x;
    out[1] += y;
    out[2] += z;
    out[3] += x * x + y * y + z * z;
    double dr = sqrt(x * x + y * y + z * z);
    int t = (flags[i] & F_A) ? 0 : 1;
    double vprev = 0.0;
    for (int b = 0; b < nb; ++b) {
      double r = rb[b], v;
      if (dr - a > r) {
        v = 0.0;
      } else if (dr + a < r) {
        v = vfull;
      } else {
        double ca = (dr * dr + a * a - r * r) / (2.0 * dr * a);
        double cb = (r * r + dr * dr - a * a) / (2.0 * r * dr);
        double va = (M_PI / 3.0) * a * a * a * (2.0 + ca) * (1.0 - ca) * (1.0 - ca);
        double vb = (M_PI / 3.0) * r * r * r * (2.0 + cb) * (1.0 - cb) * (1.0 - cb);
        v = va + vb;
      }
      out[4 + t * nb + b] += v - vprev;
      out[4 + 2 * nb + b] += v - vprev;
      vprev = v;
    }
  }
}

/* Sum over p of |r_{p+s} - r_p| for s = 0..L/2 of one chain (sd of
 * calc_sd_cp, chrana.cu:32-42), FP64. */
void orc_sdist(int L, const float *xyz, double *ds) {
  for (int s = 0; s <= L / 2; ++s) {
    double acc = 0.0;
    for (int p = 0; p + s < L; ++p) {
      if (s == 0) break;
      double dx = (double)xyz[3 * (p + s)] - xyz[3 * p];
      double dy = (double)xyz[3 * (p + s) + 1] - xyz[3 * p + 1];
      double dz = (double)xyz[3 * (p + s) + 2] - xyz[3 * p + 2];
      acc += sqrt(dx * dx + dy * dy + dz * dz);
    }
    ds[s] = acc;
  }
}

/* ------------------------------------------------------------ random walk */

/* Inverse error function by Newton iteration on erf (erf'(x) =
 * 2/sqrt(pi) exp(-x^2)), from the start 0.5 ln((1+y)/(1-y)) / 1.2; +-inf at
 * |y| >= 1. */
static double erfinv_newton(double y) {
  if (y <= -1.0) return -INFINITY;
  if (y >= 1.0) return INFINITY;
  double x = 0.5 * log((1.0 + y) / (1.0 - y)) / 1.2;
  for (int k = 0; k < 100; ++k) {
    double e = erf(x) - y, d = 1.1283791670955126 * exp(-x * x);
    if (d == 0.0) break;
    double st = e / d;
    if (st > 1.0) st = 1.0;
    if (st < -1.0) st = -1.0;
    x -= st;
    if (fabs(st) < 1e-15 * (fabs(x) > 1.0 ? fabs(x) : 1.0)) break;
  }
  return x;
}

static double u24(uint32_t x) { return (double)((x >> 8) + 1u) / 16777216.0; }

/* Confined random walk of one chain of n beads, in double
 * (chrsim::perform_random_walk, chrsim.cu:719-802), on the engine's stream:
 * attempt k draws the Philox block of counter (k, chain, 0x10057, 0x1C0DE)
 * keyed by the system seed (two uniforms for the direction, one for the bond
 * angle, one for the bond length; the first bead uses three). Sequential: an
 * attempt is accepted when the position is finite, at least mis from the wall
 * and (axis non-zero) inside the cone acos(r.a/|r||a|) <= mda; after more
 * than 1024 consecutive rejections every rejection moves back to bead
 * 1 + i*3/4 (then on to the next), the rejected candidate staying written.
 * c_b: the density of cos(bond angle) is exp(c_b cos). Returns the attempts used, or
 * -1 when max_draws ran out; *n_back (if not NULL) counts the moves back. */
long long orc_random_walk(int n, double *xyz, uint32_t k0, uint32_t k1, uint32_t chain,
                          const double *axis, double cos_mda, double R_n, double mis,
                          double c_b, double l_0, double sig_b, long long max_draws,
                          long long *n_back) {
  if (n_back) *n_back = 0;
  double la = sqrt(axis[0] * axis[0] + axis[1] * axis[1] + axis[2] * axis[2]);
  long long draw = 0;
  uint32_t o[4];
  double old[3], d_r;
  for (;;) {
    if (draw >= max_draws) return -1;
    uint32_t c[4] = {(uint32_t)draw++, chain, 0x10057u, 0x1C0DEu};
    philox10(c, k0, k1, o);
    double ct = 1.0 - 2.0 * u24(o[0]), st = sqrt(fmax(0.0, 1.0 - ct * ct));
    double ph = 2.0 * M_PI * u24(o[1]);
    old[0] = st * cos(ph);
    old[1] = st * sin(ph);
    old[2] = ct;
    d_r = (R_n - mis) * cbrt(u24(o[2]));
    for (int a = 0; a < 3; ++a) xyz[a] = d_r * old[a];
    if (la == 0.0) break;
    /* acos(r.a / (|r| |a|)) > mda rejects: r.a < cos(mda) |r| |a| */
    if (!(xyz[0] * axis[0] + xyz[1] * axis[1] + xyz[2] * axis[2] < cos_mda * d_r * la)) break;
  }
  const double one_m_e = 1.0 - exp(-2.0 * c_b);
  int att = 0;
  for (int i = 1; i < n; ++i) {
    if (draw >= max_draws) return -1;
    uint32_t c[4] = {(uint32_t)draw++, chain, 0x10057u, 0x1C0DEu};
    philox10(c, k0, k1, o);
    double ct = 1.0 - 2.0 * u24(o[0]), st = sqrt(fmax(0.0, 1.0 - ct * ct));
    double ph = 2.0 * M_PI * u24(o[1]);
    double rd[3] = {st * cos(ph), st * sin(ph), ct};
    double per[3] = {old[1] * rd[2] - old[2] * rd[1], old[2] * rd[0] - old[0] * rd[2],
                     old[0] * rd[1] - old[1] * rd[0]};
    double il = 1.0 / sqrt(per[0] * per[0] + per[1] * per[1] + per[2] * per[2]);
    double cb = 1.0 + log1p(-one_m_e * u24(o[2])) * (1.0 / c_b);
    if (cb > 1.0) cb = 1.0;
    if (cb < -1.0) cb = -1.0;
    double sb = sqrt(1.0 - cb * cb) * il;
    double lb = l_0 + sig_b * erfinv_newton(2.0 * u24(o[3]) - 1.0);
    double nd[3], *p = xyz + 3 * (size_t)i, *q = xyz + 3 * (size_t)(i - 1);
    for (int a = 0; a < 3; ++a) {
      nd[a] = cb * old[a] + sb * per[a];
      p[a] = lb * nd[a] + q[a];
    }
    int ok = isfinite(p[0]) && isfinite(p[1]) && isfinite(p[2]);
    double dr = sqrt(p[0] * p[0] + p[1] * p[1] + p[2] * p[2]);
    if ((R_n - dr) < mis) ok = 0;
    if (la != 0.0 && p[0] * axis[0] + p[1] * axis[1] + p[2] * axis[2] < cos_mda * dr * la) ok = 0;
    if (ok) {
      att = 0;
      for (int a = 0; a < 3; ++a) old[a] = nd[a];
    } else if ((att = att < (1 << 20) ? att + 1 : att) > 1024) {
      i = 1 + i * 3 / 4;
      if (n_back) ++*n_back;
    } else {
      --i;
    }
  }
  return draw;
}

int orc_max_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}
