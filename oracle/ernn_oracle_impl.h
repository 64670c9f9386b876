/*
 * CPU restatement of the ERNN finite-difference cell and its exact discrete
 * adjoint.  TEST INFRASTRUCTURE ONLY: this file is the oracle that the CUDA
 * path is compared against.  It is never linked into the product library.
 *
 * Included twice by ernn_oracle.c, once with REAL=float (the precision the
 * reference computes in) and once with REAL=double (the FP64 run of the same
 * scheme).  FN(x) appends the precision suffix.
 *
 * Reference behaviour restated here (paths inside the reference project):
 *   Parameter_inversion/Inversion_adam.py:44-51    zero-padded 3x3 stencils
 *   Parameter_inversion/Inversion_adam.py:54-106   operator, (L + f)/rho
 *   Parameter_inversion/Inversion_adam.py:240-307  leapfrog loop, history
 *   Damage_inversion/Inversion_adam.py:100-176     per-cell constants
 *   Parameter_inversion/Inversion_adam.py:447      gradient = autograd of the
 *                                                  loop; restated below as the
 *                                                  exact discrete adjoint.
 */

/* value of field a at (i, j) with the zero ghost ring outside the grid */
#define AT(a, i, j) \
  (((i) < 0 || (i) >= nx || (j) < 0 || (j) >= ny) ? (REAL)0 : (a)[(size_t)(i) * ny + (j)])

/* The three second-difference stencils of Inversion_adam.py:59-69 applied at
 * (i, j).  i runs over nx (the "x" axis of the operator), j over ny ("y").
 * w1 = h^-2, w2 = -2 h^-2, wq = h^-2 / 4, rounded as the reference rounds them
 * (a float multiple of the float h^-2). */
static inline REAL FN(dxx)(const REAL* u, int nx, int ny, int i, int j, REAL w1, REAL w2) {
  return w1 * AT(u, i - 1, j) + w2 * AT(u, i, j) + w1 * AT(u, i + 1, j);
}
static inline REAL FN(dyy)(const REAL* u, int nx, int ny, int i, int j, REAL w1, REAL w2) {
  return w1 * AT(u, i, j - 1) + w2 * AT(u, i, j) + w1 * AT(u, i, j + 1);
}
static inline REAL FN(dxy)(const REAL* u, int nx, int ny, int i, int j, REAL wq) {
  /* cross-correlation with [[.25,0,-.25],[0,0,0],[-.25,0,.25]] on the
   * (y, x)-transposed field, written back in (x, y) order */
  return wq * AT(u, i - 1, j - 1) - wq * AT(u, i + 1, j - 1) - wq * AT(u, i - 1, j + 1) +
         wq * AT(u, i + 1, j + 1);
}

/* Six constants at cell c: scalar mode uses C[0..5]; per-cell modes use
 * planes.  Order everywhere: C11, C22, C12, C16, C26, C66. */
static inline void FN(consts_at)(const OracleProblem* p, const REAL* C, const REAL* D, size_t c,
                                 size_t N, REAL k[6]) {
  int t;
  if (p->mode == ORACLE_MODE_FIELDS) {
    for (t = 0; t < 6; ++t) k[t] = C[(size_t)t * N + c];
  } else if (p->mode == ORACLE_MODE_DFIELD) {
    /* C_ij(x) = (1 - D(x)) C0_ij, evaluated as the six per-cell fields a
     * caller of the reference's spatially varying operator would pass */
    REAL s = (REAL)1 - D[c];
    for (t = 0; t < 6; ++t) k[t] = s * C[t];
  } else {
    for (t = 0; t < 6; ++t) k[t] = C[t];
  }
}

/* One application of the operator, Inversion_adam.py:54-106:
 *   Lux = C11 uxx + C66 uxyy... then (L + f) / rho. */
static void FN(apply_operator)(const OracleProblem* p, const REAL* C, const REAL* D,
                               const REAL* ux, const REAL* uy, const REAL* fx, const REAL* fy,
                               REAL rho, REAL* Lux, REAL* Luy) {
  const int nx = p->nx, ny = p->ny;
  const size_t N = (size_t)nx * ny;
  const REAL hinv2 = (REAL)(1.0 / (p->h * p->h));
  const REAL w1 = hinv2, w2 = hinv2 * (REAL)-2, wq = hinv2 * (REAL)0.25;
  long cc;
#pragma omp parallel for schedule(static)
  for (cc = 0; cc < (long)N; ++cc) {
    const int i = (int)(cc / ny), j = (int)(cc % ny);
    REAL k[6];
    FN(consts_at)(p, C, D, (size_t)cc, N, k);
    {
      const REAL C11 = k[0], C22 = k[1], C12 = k[2], C16 = k[3], C26 = k[4], C66 = k[5];
      const REAL xx_x = FN(dxx)(ux, nx, ny, i, j, w1, w2), yy_x = FN(dyy)(ux, nx, ny, i, j, w1, w2);
      const REAL xx_y = FN(dxx)(uy, nx, ny, i, j, w1, w2), yy_y = FN(dyy)(uy, nx, ny, i, j, w1, w2);
      const REAL xy_x = FN(dxy)(ux, nx, ny, i, j, wq), xy_y = FN(dxy)(uy, nx, ny, i, j, wq);
      /* Inversion_adam.py:86-98, left-to-right as Python evaluates it.  The
       * constants are float32 tensors in the reference even in its FP64 run,
       * so C12 + C66 is a float32 sum there (ref_f32_sum mirrors that). */
      const REAL c1266 = p->ref_f32_sum ? (REAL)((float)C12 + (float)C66) : C12 + C66;
      REAL lx = C11 * xx_x + C66 * yy_x + c1266 * xy_y + ((REAL)2 * C16) * xy_x +
                C16 * xx_y + C26 * yy_y;
      REAL ly = C66 * xx_y + C22 * yy_y + c1266 * xy_x + C16 * xx_x + C26 * yy_x +
                ((REAL)2 * C26) * xy_y;
      /* Inversion_adam.py:103-104 */
      Lux[cc] = (lx + (fx ? fx[cc] : (REAL)0)) / rho;
      Luy[cc] = (ly + (fy ? fy[cc] : (REAL)0)) / rho;
    }
  }
}

int FN(oracle_operator)(const OracleProblem* p, const REAL* C, const REAL* D, const REAL* ux,
                        const REAL* uy, const REAL* fx, const REAL* fy, REAL rho, REAL* Lux,
                        REAL* Luy) {
  int rc = oracle_check(p);
  if (rc) return rc;
  FN(apply_operator)(p, C, D, ux, uy, fx, fy, rho, Lux, Luy);
  return 0;
}

/* One forward step of shot s, Inversion_adam.py:264-301 (step i, 0 <= i < nt):
 *   u^{i+1} = 2 u^i - u^{i-1} + dt^2 (A u^i + f^i) / rho,
 * with f^i = signal[shot, i] * map in component src_comp.  (ux1, uy1) hold
 * u^i, (ux2, uy2) hold u^{i-1} and receive u^{i+1}; Lx, Ly, f are work
 * planes of N values. */
static void FN(fwd_step)(const OracleProblem* p, const REAL* C, const REAL* D,
                         const REAL* src_signal, const REAL* src_map, const int32_t* src_origin,
                         REAL rho, int s, int i, const REAL* ux1, const REAL* uy1, REAL* ux2,
                         REAL* uy2, REAL* Lx, REAL* Ly, REAL* f) {
  const int nx = p->nx, ny = p->ny, nt = p->nt;
  const size_t N = (size_t)nx * ny;
  const REAL dt2 = (REAL)(p->dt * p->dt);
  /* Inversion_adam.py:270-277: force = signal[i] * spatial map */
  const REAL amp = src_signal[(size_t)s * nt + i];
  const int x0 = src_origin[2 * s], y0 = src_origin[2 * s + 1];
  int a, b;
  long cc;
  memset(f, 0, N * sizeof(REAL));
  for (a = 0; a < p->src_bx; ++a)
    for (b = 0; b < p->src_by; ++b) {
      const int xi = x0 + a, yj = y0 + b;
      if (xi < 0 || xi >= nx || yj < 0 || yj >= ny) continue;
      f[(size_t)xi * ny + yj] = amp * src_map[((size_t)s * p->src_bx + a) * p->src_by + b];
    }
  FN(apply_operator)(p, C, D, ux1, uy1, p->src_comp == 0 ? f : NULL, p->src_comp == 1 ? f : NULL, rho,
                     Lx, Ly);
#pragma omp parallel for schedule(static)
  for (cc = 0; cc < (long)N; ++cc) {
    /* Inversion_adam.py:286-287, evaluated ((2u) - u') + dt^2 L */
    const REAL nxv = ((REAL)2 * ux1[cc] - ux2[cc]) + dt2 * Lx[cc];
    const REAL nyv = ((REAL)2 * uy1[cc] - uy2[cc]) + dt2 * Ly[cc];
    ux2[cc] = nxv; /* u^{i-1} slot now holds u^{i+1} */
    uy2[cc] = nyv;
  }
}

/* Inversion_adam.py:299-301: step i records u^{i+1} (ux, uy) as frame
 * i / stride when i % stride == 0 (dense history or receiver traces). */
static void FN(record_frame)(const OracleProblem* p, const int32_t* rec_idx, int s, int i,
                             const REAL* ux, const REAL* uy, REAL* out_ux, REAL* out_uy) {
  const size_t N = (size_t)p->nx * p->ny;
  const int nt_out = (p->nt + p->stride - 1) / p->stride;
  if (i % p->stride != 0) return;
  {
    const int fr = i / p->stride;
    if (p->record == ORACLE_RECORD_FIELDS) {
      memcpy(out_ux + ((size_t)s * nt_out + fr) * N, ux, N * sizeof(REAL));
      memcpy(out_uy + ((size_t)s * nt_out + fr) * N, uy, N * sizeof(REAL));
    } else {
      int r;
      for (r = 0; r < p->nrec; ++r) {
        const int32_t c = rec_idx[(size_t)s * p->nrec + r];
        out_ux[((size_t)s * nt_out + fr) * p->nrec + r] = ux[c];
        out_uy[((size_t)s * nt_out + fr) * p->nrec + r] = uy[c];
      }
    }
  }
}

/* Forward time loop, Inversion_adam.py:240-307, batched over shots that share
 * the medium: steps i = 0 .. nt-1 from u^0 = u^-1 = 0 (fwd_step), frames
 * recorded as record_frame describes.
 * If `states` is non-NULL it receives u^0..u^nt for every shot, laid out
 * [n][shot][comp][cell], which is what oracle_adjoint consumes. */
int FN(oracle_forward)(const OracleProblem* p, const REAL* C, const REAL* D,
                       const REAL* src_signal, const REAL* src_map, const int32_t* src_origin,
                       const int32_t* rec_idx, REAL rho, REAL* out_ux, REAL* out_uy,
                       REAL* states) {
  int rc = oracle_check(p);
  if (rc) return rc;
  {
    const int nt = p->nt, S = p->nshots;
    const size_t N = (size_t)p->nx * p->ny;
    REAL* buf = (REAL*)calloc(7 * N, sizeof(REAL));
    REAL *ux1 = buf, *uy1 = buf + N, *ux2 = buf + 2 * N, *uy2 = buf + 3 * N;
    REAL *Lx = buf + 4 * N, *Ly = buf + 5 * N, *f = buf + 6 * N;
    int s, i;
    if (!buf) return ORACLE_ERR_ALLOC;
    for (s = 0; s < S; ++s) {
      memset(buf, 0, 7 * N * sizeof(REAL));
      ux1 = buf; uy1 = buf + N; ux2 = buf + 2 * N; uy2 = buf + 3 * N;
      if (states) memset(states + ((size_t)0 * S + s) * 2 * N, 0, 2 * N * sizeof(REAL));
      for (i = 0; i < nt; ++i) {
        FN(fwd_step)(p, C, D, src_signal, src_map, src_origin, rho, s, i, ux1, uy1, ux2, uy2, Lx, Ly, f);
        { REAL* t = ux1; ux1 = ux2; ux2 = t; t = uy1; uy1 = uy2; uy2 = t; }
        if (states) {
          REAL* dst = states + ((size_t)(i + 1) * S + s) * 2 * N;
          memcpy(dst, ux1, N * sizeof(REAL));
          memcpy(dst + N, uy1, N * sizeof(REAL));
        }
        FN(record_frame)(p, rec_idx, s, i, ux1, uy1, out_ux, out_uy);
      }
    }
    free(buf);
  }
  return 0;
}

/* Forward time loop with checkpoints instead of every state: as
 * oracle_forward, and for every segment start i0 = j k (j = 0 .. nseg-1,
 * nseg = ceil(nt / k)) the pair (u^{i0}, u^{i0-1}) goes to
 * ckpt[j][shot][level][comp][cell] (level 0: u^{i0}, level 1: u^{i0-1}),
 * which is what oracle_adjoint_ckpt recomputes the segments from. */
int FN(oracle_forward_ckpt)(const OracleProblem* p, const REAL* C, const REAL* D,
                            const REAL* src_signal, const REAL* src_map, const int32_t* src_origin,
                            const int32_t* rec_idx, REAL rho, int k, REAL* out_ux, REAL* out_uy,
                            REAL* ckpt) {
  int rc = oracle_check(p);
  if (rc) return rc;
  if (k < 1 || !ckpt) return ORACLE_ERR_INVALID;
  {
    const int nt = p->nt, S = p->nshots;
    const size_t N = (size_t)p->nx * p->ny;
    REAL* buf = (REAL*)calloc(7 * N, sizeof(REAL));
    REAL *ux1, *uy1, *ux2, *uy2;
    REAL *Lx = buf + 4 * N, *Ly = buf + 5 * N, *f = buf + 6 * N;
    int s, i;
    if (!buf) return ORACLE_ERR_ALLOC;
    for (s = 0; s < S; ++s) {
      memset(buf, 0, 7 * N * sizeof(REAL));
      ux1 = buf; uy1 = buf + N; ux2 = buf + 2 * N; uy2 = buf + 3 * N;
      for (i = 0; i < nt; ++i) {
        if (i % k == 0) {
          REAL* dst = ckpt + (((size_t)(i / k) * S + s) * 2) * 2 * N;
          memcpy(dst, ux1, N * sizeof(REAL));
          memcpy(dst + N, uy1, N * sizeof(REAL));
          memcpy(dst + 2 * N, ux2, N * sizeof(REAL));
          memcpy(dst + 3 * N, uy2, N * sizeof(REAL));
        }
        FN(fwd_step)(p, C, D, src_signal, src_map, src_origin, rho, s, i, ux1, uy1, ux2, uy2, Lx, Ly, f);
        { REAL* t = ux1; ux1 = ux2; ux2 = t; t = uy1; uy1 = uy2; uy2 = t; }
        FN(record_frame)(p, rec_idx, s, i, ux1, uy1, out_ux, out_uy);
      }
    }
    free(buf);
  }
  return 0;
}

/* (A^T lam) for the operator above.  Each stencil is symmetric under the zero
 * ghost ring, so the transpose applies the stencils to the pointwise products
 * of the constants with lam:
 *   (A^T lam)_x = Dxx(C11 lx + C16 ly) + Dyy(C66 lx + C26 ly) + Dxy(2 C16 lx + (C12+C66) ly)
 *   (A^T lam)_y = Dxx(C16 lx + C66 ly) + Dyy(C26 lx + C22 ly) + Dxy((C12+C66) lx + 2 C26 ly)
 * Work buffer P holds the six product planes. */
static void FN(apply_transpose)(const OracleProblem* p, const REAL* C, const REAL* D,
                                const REAL* lx, const REAL* ly, REAL* P, REAL* outx,
                                REAL* outy) {
  const int nx = p->nx, ny = p->ny;
  const size_t N = (size_t)nx * ny;
  const REAL hinv2 = (REAL)(1.0 / (p->h * p->h));
  const REAL w1 = hinv2, w2 = hinv2 * (REAL)-2, wq = hinv2 * (REAL)0.25;
  long cc;
#pragma omp parallel for schedule(static)
  for (cc = 0; cc < (long)N; ++cc) {
    REAL k[6];
    FN(consts_at)(p, C, D, (size_t)cc, N, k);
    {
      const REAL C11 = k[0], C22 = k[1], C12 = k[2], C16 = k[3], C26 = k[4], C66 = k[5];
      const REAL a = lx[cc], b = ly[cc];
      P[0 * N + cc] = C11 * a + C16 * b;
      P[1 * N + cc] = C66 * a + C26 * b;
      const REAL c1266 = p->ref_f32_sum ? (REAL)((float)C12 + (float)C66) : C12 + C66;
      P[2 * N + cc] = (REAL)2 * C16 * a + c1266 * b;
      P[3 * N + cc] = C16 * a + C66 * b;
      P[4 * N + cc] = C26 * a + C22 * b;
      P[5 * N + cc] = c1266 * a + (REAL)2 * C26 * b;
    }
  }
#pragma omp parallel for schedule(static)
  for (cc = 0; cc < (long)N; ++cc) {
    const int i = (int)(cc / ny), j = (int)(cc % ny);
    outx[cc] = FN(dxx)(P + 0 * N, nx, ny, i, j, w1, w2) + FN(dyy)(P + 1 * N, nx, ny, i, j, w1, w2) +
               FN(dxy)(P + 2 * N, nx, ny, i, j, wq);
    outy[cc] = FN(dxx)(P + 3 * N, nx, ny, i, j, w1, w2) + FN(dyy)(P + 4 * N, nx, ny, i, j, w1, w2) +
               FN(dxy)(P + 5 * N, nx, ny, i, j, wq);
  }
}

/* One step of the exact discrete adjoint of oracle_forward (what
 * loss.backward() computes at Inversion_adam.py:447 /
 * Damage_inversion/Inversion_adam.py:511), shot s, m from nt down to 1.
 * With kappa = dt^2 / rho and lam^m = dL/du^m:
 *   imaging (m <= nt-1, u = u^m):  dL/dC += kappa lam^{m+1} . d(A u^m)/dC
 *   lam^m = g^m + 2 lam^{m+1} - lam^{m+2} + kappa A^T lam^{m+1}
 * g^m is the output gradient of the frame that recorded u^m.  (l1x, l1y)
 * hold lam^{m+1}, (l2x, l2y) hold lam^{m+2} and receive lam^m.  acc: 6
 * doubles (scalar constants) or 6 planes of N (per-cell modes), summed in
 * double.  tx, ty: N values each, P: 6N values of work space. */
static void FN(adj_step)(const OracleProblem* p, const REAL* C, const REAL* D, REAL rho,
                         const int32_t* rec_idx, const REAL* g_ux, const REAL* g_uy, int s, int m,
                         const REAL* ux, REAL* l1x, REAL* l1y, REAL* l2x, REAL* l2y, REAL* tx,
                         REAL* ty, REAL* P, double* acc) {
  const int nx = p->nx, ny = p->ny, nt = p->nt;
  const size_t N = (size_t)nx * ny;
  const int nt_out = (nt + p->stride - 1) / p->stride;
  const REAL dt2 = (REAL)(p->dt * p->dt);
  const REAL kappa = dt2 / rho;
  const REAL hinv2 = (REAL)(1.0 / (p->h * p->h));
  const REAL w1 = hinv2, w2 = hinv2 * (REAL)-2, wq = hinv2 * (REAL)0.25;
  const int percell = (p->mode != ORACLE_MODE_SCALAR);
  long cc;
  /* imaging term n = m: lam^{m+1} . d(A u^m)/dC (zero when m == nt).  The
   * scalar sums run over ORACLE_CHUNKS fixed chunks of cells, each summed in
   * order and the chunks in order: the result does not depend on the number
   * of threads. */
  if (m <= nt - 1 && ux) {
    const REAL* uy = ux + N;
    double part[ORACLE_CHUNKS][6];
    const long chunk = ((long)N + ORACLE_CHUNKS - 1) / ORACLE_CHUNKS;
    long ch;
#pragma omp parallel for schedule(static)
    for (ch = 0; ch < ORACLE_CHUNKS; ++ch) {
      double sum[6] = {0, 0, 0, 0, 0, 0};
      const long c0 = ch * chunk, c1 = (ch + 1) * chunk < (long)N ? (ch + 1) * chunk : (long)N;
      int q;
      long c;
      for (c = c0; c < c1; ++c) {
        const int i = (int)(c / ny), j = (int)(c % ny);
        const double a = l1x[c], b = l1y[c];
        const double xx_x = FN(dxx)(ux, nx, ny, i, j, w1, w2), yy_x = FN(dyy)(ux, nx, ny, i, j, w1, w2);
        const double xx_y = FN(dxx)(uy, nx, ny, i, j, w1, w2), yy_y = FN(dyy)(uy, nx, ny, i, j, w1, w2);
        const double xy_x = FN(dxy)(ux, nx, ny, i, j, wq), xy_y = FN(dxy)(uy, nx, ny, i, j, wq);
        double g[6];
        g[0] = a * xx_x;                                   /* dLux/dC11 */
        g[1] = b * yy_y;                                   /* dLuy/dC22 */
        g[2] = a * xy_y + b * xy_x;                        /* C12 */
        g[3] = a * (2.0 * xy_x + xx_y) + b * xx_x;         /* C16 */
        g[4] = a * yy_y + b * (yy_x + 2.0 * xy_y);         /* C26 */
        g[5] = a * (yy_x + xy_y) + b * (xx_y + xy_x);      /* C66 */
        if (percell) {
          for (q = 0; q < 6; ++q) acc[(size_t)q * N + c] += (double)kappa * g[q];
        } else {
          for (q = 0; q < 6; ++q) sum[q] += g[q];
        }
      }
      for (q = 0; q < 6; ++q) part[ch][q] = sum[q];
    }
    if (!percell) {
      int q;
      for (q = 0; q < 6; ++q) {
        double v = 0.0;
        for (ch = 0; ch < ORACLE_CHUNKS; ++ch) v += part[ch][q];
        acc[q] += (double)kappa * v;
      }
    }
  }
  /* lam^m = 2 lam^{m+1} - lam^{m+2} + kappa A^T lam^{m+1} + g^m */
  FN(apply_transpose)(p, C, D, l1x, l1y, P, tx, ty);
#pragma omp parallel for schedule(static)
  for (cc = 0; cc < (long)N; ++cc) {
    l2x[cc] = ((REAL)2 * l1x[cc] - l2x[cc]) + kappa * tx[cc];
    l2y[cc] = ((REAL)2 * l1y[cc] - l2y[cc]) + kappa * ty[cc];
  }
  if ((m - 1) % p->stride == 0) {
    const int fr = (m - 1) / p->stride;
    if (p->record == ORACLE_RECORD_FIELDS) {
      const REAL* gx = g_ux + ((size_t)s * nt_out + fr) * N;
      const REAL* gy = g_uy + ((size_t)s * nt_out + fr) * N;
      for (cc = 0; cc < (long)N; ++cc) { l2x[cc] += gx[cc]; l2y[cc] += gy[cc]; }
    } else {
      int r;
      for (r = 0; r < p->nrec; ++r) {
        const int32_t c = rec_idx[(size_t)s * p->nrec + r];
        l2x[c] += g_ux[((size_t)s * nt_out + fr) * p->nrec + r];
        l2y[c] += g_uy[((size_t)s * nt_out + fr) * p->nrec + r];
      }
    }
  }
}

/* Gradient outputs from the accumulators of adj_step:
 *   SCALAR: grad_C[6]   (C11, C22, C12, C16, C26, C66)
 *   FIELDS: grad_C[6*N] per-cell planes
 *   DFIELD: grad_D[N]   dL/dD = -sum_t C0_t dL/dC_t(x); grad_C (may be NULL)
 *           dL/dC0_t = sum_x (1 - D(x)) dL/dC_t(x) */
static void FN(finish_gradient)(const OracleProblem* p, const REAL* C, const REAL* D, const double* acc,
                                double* grad_C, double* grad_D) {
  const size_t N = (size_t)p->nx * p->ny;
  int t;
  if (p->mode == ORACLE_MODE_SCALAR) {
    for (t = 0; t < 6; ++t) grad_C[t] = acc[t];
  } else if (p->mode == ORACLE_MODE_FIELDS) {
    memcpy(grad_C, acc, 6 * N * sizeof(double));
  } else {
    size_t c;
    if (grad_C) for (t = 0; t < 6; ++t) grad_C[t] = 0.0;
    for (c = 0; c < N; ++c) {
      double v = 0.0;
      for (t = 0; t < 6; ++t) v -= (double)C[t] * acc[(size_t)t * N + c];
      grad_D[c] = v;
      if (grad_C)
        for (t = 0; t < 6; ++t) grad_C[t] += (1.0 - (double)D[c]) * acc[(size_t)t * N + c];
    }
  }
}

/* Exact discrete adjoint of oracle_forward over every step (adj_step for
 * m = nt .. 1), reading the states u^0..u^nt that oracle_forward stored. */
int FN(oracle_adjoint)(const OracleProblem* p, const REAL* C, const REAL* D, REAL rho,
                       const int32_t* rec_idx, const REAL* states, const REAL* g_ux,
                       const REAL* g_uy, double* grad_C, double* grad_D) {
  int rc = oracle_check(p);
  if (rc) return rc;
  {
    const int nt = p->nt, S = p->nshots;
    const size_t N = (size_t)p->nx * p->ny;
    const int percell = (p->mode != ORACLE_MODE_SCALAR);
    REAL* buf = (REAL*)calloc(12 * N, sizeof(REAL));
    double* acc = (double*)calloc(percell ? 6 * N : 6, sizeof(double));
    REAL *l1x, *l1y, *l2x, *l2y, *tx = buf + 4 * N, *ty = buf + 5 * N, *P = buf + 6 * N;
    int s, m;
    if (!buf || !acc) { free(buf); free(acc); return ORACLE_ERR_ALLOC; }
    for (s = 0; s < S; ++s) {
      memset(buf, 0, 4 * N * sizeof(REAL));
      l1x = buf; l1y = buf + N; l2x = buf + 2 * N; l2y = buf + 3 * N;
      for (m = nt; m >= 1; --m) {
        const REAL* ux = m <= nt - 1 ? states + ((size_t)m * S + s) * 2 * N : NULL;
        FN(adj_step)(p, C, D, rho, rec_idx, g_ux, g_uy, s, m, ux, l1x, l1y, l2x, l2y, tx, ty, P, acc);
        { REAL* q = l1x; l1x = l2x; l2x = q; q = l1y; l1y = l2y; l2y = q; }
      }
    }
    FN(finish_gradient)(p, C, D, acc, grad_C, grad_D);
    free(buf);
    free(acc);
  }
  return 0;
}

/* The same adjoint from the checkpoints of oracle_forward_ckpt (interval
 * k): per shot, segments j = nseg-1 .. 0 are recomputed from their pair
 * (u^{jk}, u^{jk-1}) into a buffer of k states, then m runs from the
 * segment's top, min((j+1) k, nt), down to j k + 1.  Memory: k states and
 * the checkpoints instead of nt + 1 states; the arithmetic is the same as
 * oracle_forward followed by oracle_adjoint. */
int FN(oracle_adjoint_ckpt)(const OracleProblem* p, const REAL* C, const REAL* D,
                            const REAL* src_signal, const REAL* src_map, const int32_t* src_origin,
                            const int32_t* rec_idx, REAL rho, int k, const REAL* ckpt,
                            const REAL* g_ux, const REAL* g_uy, double* grad_C, double* grad_D) {
  int rc = oracle_check(p);
  if (rc) return rc;
  if (k < 1 || !ckpt) return ORACLE_ERR_INVALID;
  {
    const int nt = p->nt, S = p->nshots;
    const int nseg = (nt + k - 1) / k;
    const size_t N = (size_t)p->nx * p->ny;
    const int percell = (p->mode != ORACLE_MODE_SCALAR);
    REAL* buf = (REAL*)calloc(12 * N, sizeof(REAL));
    REAL* fwd = (REAL*)calloc(7 * N, sizeof(REAL));
    REAL* seg = (REAL*)calloc((size_t)k * 2 * N, sizeof(REAL));  /* u^{jk+1} .. u^{jk+k} */
    double* acc = (double*)calloc(percell ? 6 * N : 6, sizeof(double));
    REAL *l1x, *l1y, *l2x, *l2y, *tx = buf + 4 * N, *ty = buf + 5 * N, *P = buf + 6 * N;
    int s, j, m, i;
    if (!buf || !fwd || !seg || !acc) {
      free(buf); free(fwd); free(seg); free(acc);
      return ORACLE_ERR_ALLOC;
    }
    for (s = 0; s < S; ++s) {
      memset(buf, 0, 4 * N * sizeof(REAL));
      l1x = buf; l1y = buf + N; l2x = buf + 2 * N; l2y = buf + 3 * N;
      for (j = nseg - 1; j >= 0; --j) {
        const int i0 = j * k, i1 = (j + 1) * k < nt ? (j + 1) * k : nt;
        REAL *ux1 = fwd, *uy1 = fwd + N, *ux2 = fwd + 2 * N, *uy2 = fwd + 3 * N;
        const REAL* cp = ckpt + (((size_t)j * S + s) * 2) * 2 * N;
        memcpy(fwd, cp, 4 * N * sizeof(REAL));
        for (i = i0; i < i1; ++i) {
          FN(fwd_step)(p, C, D, src_signal, src_map, src_origin, rho, s, i, ux1, uy1, ux2, uy2,
                       fwd + 4 * N, fwd + 5 * N, fwd + 6 * N);
          { REAL* t = ux1; ux1 = ux2; ux2 = t; t = uy1; uy1 = uy2; uy2 = t; }
          memcpy(seg + (size_t)(i - i0) * 2 * N, ux1, N * sizeof(REAL));
          memcpy(seg + (size_t)(i - i0) * 2 * N + N, uy1, N * sizeof(REAL));
        }
        for (m = i1; m >= i0 + 1; --m) {
          const REAL* ux = m <= nt - 1 ? seg + (size_t)(m - 1 - i0) * 2 * N : NULL;
          FN(adj_step)(p, C, D, rho, rec_idx, g_ux, g_uy, s, m, ux, l1x, l1y, l2x, l2y, tx, ty, P, acc);
          { REAL* q = l1x; l1x = l2x; l2x = q; q = l1y; l1y = l2y; l2y = q; }
        }
      }
    }
    FN(finish_gradient)(p, C, D, acc, grad_C, grad_D);
    free(buf);
    free(fwd);
    free(seg);
    free(acc);
  }
  return 0;
}

#undef AT
