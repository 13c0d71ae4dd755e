/*
 * Precision-generic body of the oracle (included twice by ccp_oracle.c with
 * REAL = double and REAL = float). Test infrastructure only.
 */

typedef struct {
  REAL x, y, z;
} SFX(v3);

static inline SFX(v3) SFX(sub)(SFX(v3) a, SFX(v3) b) {
  SFX(v3) r = {a.x - b.x, a.y - b.y, a.z - b.z};
  return r;
}
static inline REAL SFX(dot)(SFX(v3) a, SFX(v3) b) { return a.x * b.x + a.y * b.y + a.z * b.z; }

typedef struct {
  int pot, bend_all;
  REAL k_e, l_0, k_b, e_att, e_rep, rc_rep, rc_att, e_w, rc_w, e_l, lco, lbs_depth, k_icg,
      rc_icg, dt, sd, max_step;
  REAL R_n, R_o, R_b, noc, boc, nod, bod, d_m, csl;
} SFX(model);

/* Deterministic displacement of one stage limited to max_step (> 0); the
 * baseline preset's stabiliser of the WCA core at dt = 1e-3 (not in ccp). */
static inline void SFX(cap_step)(REAL *dx, REAL *dy, REAL *dz, REAL max_step) {
  if (max_step <= 0) return;
  REAL m2 = *dx * *dx + *dy * *dy + *dz * *dz;
  if (m2 > max_step * max_step) {
    REAL k = max_step / SQRT(m2);
    *dx *= k; *dy *= k; *dz *= k;
  }
}

static SFX(model) SFX(make_model)(const double *ff, const double *geo) {
  SFX(model) m;
  m.pot = (int)ff[FF_POT];
  m.bend_all = (int)ff[FF_BEND_ALL];
  m.k_e = (REAL)ff[FF_KE];
  m.l_0 = (REAL)ff[FF_L0];
  m.k_b = (REAL)ff[FF_KB];
  m.e_att = (REAL)ff[FF_EATT];
  m.e_rep = (REAL)ff[FF_EREP];
  m.rc_rep = (REAL)ff[FF_RCREP];
  m.rc_att = (REAL)ff[FF_RCATT];
  m.e_w = (REAL)ff[FF_EW];
  m.rc_w = (REAL)ff[FF_RCW];
  m.e_l = (REAL)ff[FF_EL];
  m.lco = (REAL)ff[FF_LCO];
  m.lbs_depth = (REAL)ff[FF_LBSDEPTH];
  m.k_icg = (REAL)ff[FF_KICG];
  m.rc_icg = (REAL)ff[FF_RCICG];
  m.dt = (REAL)ff[FF_DT];
  m.sd = (REAL)ff[FF_SD];
  m.max_step = (REAL)ff[FF_MAXSTEP];
  /* cngeom (chrdat.cu:13-18) */
  double R_n = geo[G_RN], R_o = geo[G_RO], R_b = geo[G_RB];
  double noc = cos(asin(R_o / R_n)), boc = cos(asin(R_o / R_b));
  double nod = sqrt(R_n * R_n - R_o * R_o), bod = sqrt(R_b * R_b - R_o * R_o);
  m.R_n = (REAL)R_n;
  m.R_o = (REAL)R_o;
  m.R_b = (REAL)R_b;
  m.noc = (REAL)noc;
  m.boc = (REAL)boc;
  m.nod = (REAL)nod;
  m.bod = (REAL)bod;
  m.d_m = (REAL)(nod + bod + R_b);
  m.csl = (REAL)geo[G_CSL];
  return m;
}

/* a^2 + b^2 + c^2 - k (k = kh + kl) with error-free products and sums, so
 * that the result keeps full relative precision when the sum is close to k
 * (bond lengths near l_0, beads near the wall). */
static inline REAL SFX(sq3_minus)(REAL a, REAL b, REAL c, REAL kh, REAL kl) {
  REAL pa = a * a, ea = fma(a, a, -pa);
  REAL pb = b * b, eb = fma(b, b, -pb);
  REAL pc = c * c, ec = fma(c, c, -pc);
  REAL s1 = pa + pb, t1 = s1 - pa, e1 = (pa - (s1 - t1)) + (pb - t1);
  REAL s2 = s1 + pc, t2 = s2 - s1, e2 = (s1 - (s2 - t2)) + (pc - t2);
  REAL s3 = s2 - kh, t3 = s3 - s2, e3 = (s2 - (s3 - t3)) + (-kh - t3);
  return s3 + (((ea + eb) + (ec + e1)) + ((e2 + e3) - kl));
}

/* Pair force coefficient c, F_i += c (r_i - r_j) (chrsim.cu:174-198), for the
 * pair vector v of length d. */
static inline REAL SFX(pair_c)(SFX(v3) v, REAL d, int hh, const SFX(model) * m, int mode) {
  if (mode == MODE_ICG) {
    if (d > m->rc_icg) return 0;
    return m->k_icg * (3 * m->rc_icg - 3 * d);
  }
  if (m->pot == POT_WF) {
    if (d > m->rc_att) return 0;
    if (!hh && d > m->rc_rep) return 0;
    REAL d2 = d * d;
#if ORC_ACCURATE
    REAL i2 = 1 / d2, i4 = i2 * i2;
    return m->e_att * 6 * ((d2 - 4) * fma((REAL)3, d2, (REAL)-4)) * (i4 * i4);
#else
    return m->e_att * (18 * d2 * d2 - 96 * d2 + 96) / (d2 * d2 * d2 * d2);
#endif
  }
  REAL rc = hh ? m->rc_att : m->rc_rep;
  if (d > rc) return 0;
  REAL e = hh ? m->e_att : m->e_rep;
  REAL i2 = 1 / (d * d), i6 = i2 * i2 * i2;
#if ORC_ACCURATE
  /* the repulsive class near its cutoff 2^(1/6), the force's zero:
   * 2 d^-6 - 1 = -(d^2 - 2^(1/3)) (d^4 + 2^(1/3) d^2 + 2^(2/3)) d^-6 from an
   * error-free d^2 - 2^(1/3) (the engine's lj_coef) */
  if (!hh) {
    const REAL z2h = (REAL)1.259921074e+00, z2l = (REAL)-2.401870169e-08;
    REAL d2 = d * d;
    REAL t = SFX(sq3_minus)(v.x, v.y, v.z, z2h, z2l);
    REAL q = fma(d2, d2 + z2h, (REAL)1.587401032e+00);
    return 24 * e * (i6 * i2) * (-t * q * i6);
  }
  return 24 * e * (i6 * i2) * fma((REAL)2, i6, (REAL)-1);
#else
  return 24 * e * (2 * i6 * i6 - i6) * i2;
#endif
}

/* Wall force (chrsim.cu:79-170). */
static inline SFX(v3) SFX(wall)(SFX(v3) r, const SFX(model) * m, int mode) {
  SFX(v3) v, f = {0, 0, 0};
  REAL d_r;
#if ORC_ACCURATE
  /* R/d - 1 = (R^2 - d^2) / ((R + d) d) with R^2 - d^2 free of cancellation */
#define ORC_RM1(R, a, b, c, dd) \
  (-SFX(sq3_minus)(a, b, c, (R) * (R), fma(R, R, -(R) * (R))) / (((R) + (dd)) * (dd)))
#else
#define ORC_RM1(R, a, b, c, dd) ((R) / (dd) - 1)
#endif
  if (mode == MODE_ICG) {
    d_r = SQRT(SFX(dot)(r, r));
    REAL k = -ORC_RM1(m->R_n, r.x, r.y, r.z, d_r);
    v.x = r.x * k; v.y = r.y * k; v.z = r.z * k;
  } else if (r.z < m->nod) {
    d_r = SQRT(SFX(dot)(r, r));
    if (r.z / d_r < m->noc) {
      REAL k = -ORC_RM1(m->R_n, r.x, r.y, r.z, d_r);
      v.x = r.x * k; v.y = r.y * k; v.z = r.z * k;
    } else {
      d_r = SQRT(r.x * r.x + r.y * r.y);
      REAL k = ORC_RM1(m->R_o, r.x, r.y, (REAL)0, d_r);
      v.x = -r.x * k;
      v.y = -r.y * k;
      v.z = r.z - m->nod;
    }
  } else {
    SFX(v3) q = {r.x, r.y, r.z - (m->nod + m->bod)};
    d_r = SQRT(SFX(dot)(q, q));
    if (-q.z / d_r < m->boc) {
      REAL k = -ORC_RM1(m->R_b, q.x, q.y, q.z, d_r);
      v.x = q.x * k; v.y = q.y * k; v.z = q.z * k;
    } else {
      d_r = SQRT(q.x * q.x + q.y * q.y);
      REAL k = ORC_RM1(m->R_o, q.x, q.y, (REAL)0, d_r);
      v.x = -q.x * k;
      v.y = -q.y * k;
      v.z = q.z + m->bod;
    }
  }
#undef ORC_RM1
  REAL d = SQRT(SFX(dot)(v, v));
  if (!isfinite(d)) return f;
  /* the relaxation wall is ccp's calc_wpf: Wang-Frenkel, eps = 1, cutoff rco */
  int wf = (mode == MODE_ICG) || (m->pot == POT_WF);
  REAL ew = (mode == MODE_ICG) ? 1 : m->e_w;
  if (d > ((mode == MODE_ICG) ? (REAL)1.154701 : m->rc_w)) return f;
  REAL c;
  if (wf) {
    REAL d2 = d * d;
#if ORC_ACCURATE
    REAL i2 = 1 / d2, i4 = i2 * i2;
    c = ew * 6 * ((d2 - 4) * fma((REAL)3, d2, (REAL)-4)) * (i4 * i4);
#else
    c = ew * (18 * d2 * d2 - 96 * d2 + 96) / (d2 * d2 * d2 * d2);
#endif
  } else {
    REAL i2 = 1 / (d * d), i6 = i2 * i2 * i2;
#if ORC_ACCURATE
    c = 24 * m->e_w * (i6 * i2) * fma((REAL)2, i6, (REAL)-1);
#else
    c = 24 * m->e_w * (2 * i6 * i6 - i6) * i2;
#endif
  }
  f.x = c * v.x; f.y = c * v.y; f.z = c * v.z;
  return f;
}

/* Bonded + bending force of bead i (calc_bf, chrsim.cu:13-76): chain limits
 * lim_l = head + 2, lim_u = end; bond b (0..3) joins i+b-2 and i+b-1. */
static inline SFX(v3) SFX(bonded)(const SFX(v3) * r, const uint32_t *flags, int i, int head,
                                  int end, const SFX(model) * m) {
  SFX(v3) vec[4];
  REAL il[4], cs[3];
  int lim_l = head + 2, lim_u = end;
  for (int b = 0; b < 4; ++b) {
    if (i + b >= lim_l && i + b <= lim_u) {
      vec[b] = SFX(sub)(r[i + b - 1], r[i + b - 2]);
      il[b] = RSQRT(SFX(dot)(vec[b], vec[b]));
    } else {
      vec[b].x = vec[b].y = vec[b].z = 0;
      il[b] = 0;
    }
  }
  for (int c = 0; c < 3; ++c) cs[c] = SFX(dot)(vec[c + 1], vec[c]) * il[c + 1] * il[c];
  SFX(v3) f;
#if ORC_ACCURATE
  /* 1 - l_0 / d = (d^2 - l_0^2) / ((d + l_0) d) */
  REAL l2h = m->l_0 * m->l_0, l2l = fma(m->l_0, m->l_0, -l2h);
  /* residuals of the coordinate differences (TwoSum), so d^2 - l_0^2 is
   * formed from the exact bond vector */
  REAL s1 = 0, s2 = 0;
  for (int b = 1; b <= 2; ++b) {
    if (il[b] == 0) continue;
    const REAL *pa = &r[i + b - 1].x, *pb = &r[i + b - 2].x, *hv = &vec[b].x;
    REAL corr = 0;
    for (int k = 0; k < 3; ++k) {
      REAL t = hv[k] - pa[k];
      REAL lo = (pa[k] - (hv[k] - t)) + (-pb[k] - t);
      corr += hv[k] * lo;
    }
    REAL s = SFX(sq3_minus)(hv[0], hv[1], hv[2], l2h, l2l) + 2 * corr;
    if (b == 1) s1 = s; else s2 = s;
  }
  REAL dd1 = SQRT(SFX(dot)(vec[1], vec[1])), dd2 = SQRT(SFX(dot)(vec[2], vec[2]));
  REAL a1 = (il[1] == 0) ? 0 : m->k_e * (s1 / (dd1 + m->l_0)) * il[1];
  REAL a2 = (il[2] == 0) ? 0 : m->k_e * (s2 / (dd2 + m->l_0)) * il[2];
#else
  REAL a2 = m->k_e * (1 - m->l_0 * il[2]), a1 = m->k_e * (1 - m->l_0 * il[1]);
#endif
  f.x = a2 * vec[2].x - a1 * vec[1].x;
  f.y = a2 * vec[2].y - a1 * vec[1].y;
  f.z = a2 * vec[2].z - a1 * vec[1].z;
  if (m->bend_all || (flags[i] & F_A)) {
    REAL kb = m->k_b;
#define ORC_ADD(c, v) do { f.x += kb * (c) * (v).x; f.y += kb * (c) * (v).y; f.z += kb * (c) * (v).z; } while (0)
    ORC_ADD(il[1] * il[0], vec[0]);
    ORC_ADD(-cs[0] * il[1] * il[1], vec[1]);
    ORC_ADD(il[1] * il[2], vec[2]);
    ORC_ADD(-cs[1] * il[1] * il[1], vec[1]);
    ORC_ADD(-il[2] * il[1], vec[1]);
    ORC_ADD(cs[1] * il[2] * il[2], vec[2]);
    ORC_ADD(-il[2] * il[3], vec[3]);
    ORC_ADD(cs[2] * il[2] * il[2], vec[2]);
#undef ORC_ADD
  }
  return f;
}

/* LBS binding on an A/LAD bead (calc_lpf, chrsim.cu:202-212). */
static inline void SFX(lbs_add)(SFX(v3) ri, SFX(v3) l, const SFX(model) * m, SFX(v3) * f) {
  SFX(v3) v = SFX(sub)(ri, l);
  REAL d = SQRT(SFX(dot)(v, v));
  if (d > m->lco) return;
  REAL nd = d / m->lco, d2 = nd * nd;
  REAL c = m->e_l * (8 / (3 * m->lco * m->lco)) * (d2 * d2 * d2 - 1);
  f->x += c * v.x; f->y += c * v.y; f->z += c * v.z;
}

static void SFX(chain_limits)(int n, const uint32_t *flags, int *head, int *end) {
  int h = 0;
  for (int i = 0; i < n; ++i) {
    if (flags[i] & F_HEAD) h = i;
    head[i] = h;
  }
  int e = n;
  for (int i = n - 1; i >= 0; --i) {
    end[i] = e;
    if (flags[i] & F_HEAD) e = i;
  }
}

/* ---------------------------------------------------------------- cell list */

typedef struct {
  int cps, nc;
  int *start, *idx;
} SFX(cells);

static int SFX(cell_coord)(REAL v, const SFX(model) * m, int cps) {
  REAL c = floor(v / m->csl) + (REAL)(cps / 2);
  if (!(c >= 0)) return 0;
  if (c >= cps) return cps - 1;
  return (int)c;
}

static void SFX(build_cells)(int n, const SFX(v3) * r, const SFX(model) * m, SFX(cells) * g) {
  int cps = 2 * (int)ceil((double)m->d_m / (double)m->csl);
  if (cps < 2) cps = 2;
  g->cps = cps;
  g->nc = cps * cps * cps;
  g->start = (int *)calloc((size_t)g->nc + 1, sizeof(int));
  g->idx = (int *)malloc(sizeof(int) * (size_t)(n > 0 ? n : 1));
  int *key = (int *)malloc(sizeof(int) * (size_t)(n > 0 ? n : 1));
  for (int i = 0; i < n; ++i) {
    int cx = SFX(cell_coord)(r[i].x, m, cps), cy = SFX(cell_coord)(r[i].y, m, cps),
        cz = SFX(cell_coord)(r[i].z, m, cps);
    key[i] = (cz * cps + cy) * cps + cx;
    g->start[key[i] + 1]++;
  }
  for (int c = 0; c < g->nc; ++c) g->start[c + 1] += g->start[c];
  int *fill = (int *)malloc(sizeof(int) * (size_t)g->nc);
  memcpy(fill, g->start, sizeof(int) * (size_t)g->nc);
  for (int i = 0; i < n; ++i) g->idx[fill[key[i]]++] = i;
  free(fill);
  free(key);
}

static void SFX(free_cells)(SFX(cells) * g) {
  free(g->start);
  free(g->idx);
}

/* Total force of every bead. use_cells = 0: all pairs; 1: cell list. */
static void SFX(forces_core)(int n, const SFX(v3) * r, const uint32_t *flags, int n_l,
                             const SFX(v3) * lbs, const SFX(model) * m, int mode, int use_cells,
                             const int *head, const int *end, SFX(v3) * out, REAL *absum) {
  SFX(cells) g = {0, 0, NULL, NULL};
  if (use_cells) SFX(build_cells)(n, r, m, &g);
#pragma omp parallel for schedule(dynamic, 256)
  for (int i = 0; i < n; ++i) {
    SFX(v3) f = SFX(bonded)(r, flags, i, head[i], end[i], m);
    SFX(v3) w = SFX(wall)(r[i], m, mode);
    REAL sa = SQRT(SFX(dot)(f, f)) + SQRT(SFX(dot)(w, w));
    f.x += w.x; f.y += w.y; f.z += w.z;
    SFX(v3) ri = r[i];
    int ai = (flags[i] & F_A) != 0;
    if (use_cells) {
      int cps = g.cps;
      int cx = SFX(cell_coord)(ri.x, m, cps), cy = SFX(cell_coord)(ri.y, m, cps),
          cz = SFX(cell_coord)(ri.z, m, cps);
      for (int z = cz - 1; z <= cz + 1; ++z)
        for (int y = cy - 1; y <= cy + 1; ++y)
          for (int x = cx - 1; x <= cx + 1; ++x) {
            if (x < 0 || y < 0 || z < 0 || x >= cps || y >= cps || z >= cps) continue;
            int c = (z * cps + y) * cps + x;
            for (int k = g.start[c]; k < g.start[c + 1]; ++k) {
              int j = g.idx[k];
              if (abs(i - j) <= 1) continue;
              SFX(v3) v = SFX(sub)(ri, r[j]);
              REAL d = SQRT(SFX(dot)(v, v));
              REAL c2 = SFX(pair_c)(v, d, ai && (flags[j] & F_A), m, mode);
              f.x += c2 * v.x; f.y += c2 * v.y; f.z += c2 * v.z;
              sa += fabs(c2) * d;
            }
          }
    } else {
      for (int j = 0; j < n; ++j) {
        if (abs(i - j) <= 1) continue;
        SFX(v3) v = SFX(sub)(ri, r[j]);
        REAL d = SQRT(SFX(dot)(v, v));
        REAL c2 = SFX(pair_c)(v, d, ai && (flags[j] & F_A), m, mode);
        f.x += c2 * v.x; f.y += c2 * v.y; f.z += c2 * v.z;
        sa += fabs(c2) * d;
      }
    }
    if (mode == MODE_DST && (flags[i] & F_LAD))
      for (int l = 0; l < n_l; ++l) {
        SFX(v3) g0 = f;
        SFX(lbs_add)(ri, lbs[l], m, &f);
        SFX(v3) dg = SFX(sub)(f, g0);
        sa += SQRT(SFX(dot)(dg, dg));
      }
    out[i] = f;
    if (absum) absum[i] = sa;
  }
  if (use_cells) SFX(free_cells)(&g);
}

/* Forces of one system at float positions; out = 3 doubles per bead. */
void SFX(orc_forces)(int n, const float *xyz, const uint32_t *flags, int n_l, const float *lxyz,
                     const double *ff, const double *geo, int mode, int use_cells, double *out,
                     double *out_abs) {
  SFX(model) m = SFX(make_model)(ff, geo);
  SFX(v3) *r = (SFX(v3) *)malloc(sizeof(SFX(v3)) * (size_t)(n + 1));
  SFX(v3) *l = (SFX(v3) *)malloc(sizeof(SFX(v3)) * (size_t)(n_l + 1));
  SFX(v3) *f = (SFX(v3) *)malloc(sizeof(SFX(v3)) * (size_t)(n + 1));
  int *head = (int *)malloc(sizeof(int) * (size_t)(n + 1)), *end = (int *)malloc(sizeof(int) * (size_t)(n + 1));
  for (int i = 0; i < n; ++i) {
    r[i].x = xyz[3 * i]; r[i].y = xyz[3 * i + 1]; r[i].z = xyz[3 * i + 2];
  }
  for (int i = 0; i < n_l; ++i) {
    l[i].x = lxyz[3 * i]; l[i].y = lxyz[3 * i + 1]; l[i].z = lxyz[3 * i + 2];
  }
  REAL *sa = (REAL *)malloc(sizeof(REAL) * (size_t)(n + 1));
  SFX(chain_limits)(n, flags, head, end);
  SFX(forces_core)(n, r, flags, n_l, l, &m, mode, use_cells, head, end, f, sa);
  for (int i = 0; i < n; ++i) {
    out[3 * i] = f[i].x; out[3 * i + 1] = f[i].y; out[3 * i + 2] = f[i].z;
    if (out_abs) out_abs[i] = sa[i];
  }
  free(r); free(l); free(f); free(head); free(end); free(sa);
}

/* Stochastic Heun steps of one system (chrsim.cu:365-416) with the Philox
 * noise of bead i at step s, the same sd z in both stages (chrsim.cu:387,
 * :415). xyz: float positions in; out: REAL positions after nsteps (doubles). */
void SFX(orc_run)(int n, const float *xyz, const uint32_t *flags, int n_l, const float *lxyz,
                  const double *ff, const double *geo, uint32_t k0, uint32_t k1, uint64_t step0,
                  int nsteps, int mode, double *out) {
  SFX(model) m = SFX(make_model)(ff, geo);
  size_t sz = sizeof(SFX(v3)) * (size_t)(n + 1);
  SFX(v3) *r = (SFX(v3) *)malloc(sz), *er = (SFX(v3) *)malloc(sz);
  SFX(v3) *f1 = (SFX(v3) *)malloc(sz), *f2 = (SFX(v3) *)malloc(sz), *rn = (SFX(v3) *)malloc(sz);
  SFX(v3) *l = (SFX(v3) *)malloc(sizeof(SFX(v3)) * (size_t)(n_l + 1));
  int *head = (int *)malloc(sizeof(int) * (size_t)(n + 1)), *end = (int *)malloc(sizeof(int) * (size_t)(n + 1));
  for (int i = 0; i < n; ++i) {
    r[i].x = xyz[3 * i]; r[i].y = xyz[3 * i + 1]; r[i].z = xyz[3 * i + 2];
  }
  for (int i = 0; i < n_l; ++i) {
    l[i].x = lxyz[3 * i]; l[i].y = lxyz[3 * i + 1]; l[i].z = lxyz[3 * i + 2];
  }
  SFX(chain_limits)(n, flags, head, end);
  for (int s = 0; s < nsteps; ++s) {
    uint64_t step = step0 + (uint64_t)s;
#pragma omp parallel for schedule(static)
    for (int i = 0; i < n; ++i) {
      double z[3] = {0, 0, 0};
      if (mode == MODE_DST && m.sd > 0) orc_noise((uint32_t)i, step, k0, k1, z);
      rn[i].x = m.sd * (REAL)z[0]; rn[i].y = m.sd * (REAL)z[1]; rn[i].z = m.sd * (REAL)z[2];
    }
    SFX(forces_core)(n, r, flags, n_l, l, &m, mode, 1, head, end, f1, NULL);
#pragma omp parallel for schedule(static)
    for (int i = 0; i < n; ++i) {
      REAL dx = f1[i].x * m.dt, dy = f1[i].y * m.dt, dz = f1[i].z * m.dt;
      SFX(cap_step)(&dx, &dy, &dz, m.max_step);
      er[i].x = r[i].x + dx + rn[i].x;
      er[i].y = r[i].y + dy + rn[i].y;
      er[i].z = r[i].z + dz + rn[i].z;
    }
    SFX(forces_core)(n, er, flags, n_l, l, &m, mode, 1, head, end, f2, NULL);
    REAL h = (REAL)0.5 * m.dt;
#pragma omp parallel for schedule(static)
    for (int i = 0; i < n; ++i) {
      REAL dx = (f1[i].x + f2[i].x) * h, dy = (f1[i].y + f2[i].y) * h, dz = (f1[i].z + f2[i].z) * h;
      SFX(cap_step)(&dx, &dy, &dz, m.max_step);
      r[i].x = r[i].x + dx + rn[i].x;
      r[i].y = r[i].y + dy + rn[i].y;
      r[i].z = r[i].z + dz + rn[i].z;
    }
  }
  for (int i = 0; i < n; ++i) {
    out[3 * i] = r[i].x; out[3 * i + 1] = r[i].y; out[3 * i + 2] = r[i].z;
  }
  free(r); free(er); free(f1); free(f2); free(rn); free(l); free(head); free(end);
}
