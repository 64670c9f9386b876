/*
 * CPU restatement of the ERNN finite-difference cell and its exact discrete
 * adjoint.  TEST INFRASTRUCTURE ONLY: this file is the checker that the CUDA
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

/* Forward time loop, Inversion_adam.py:240-307, batched over shots that share
 * the medium.  Step i (0 <= i < nt) computes
 *   u^{i+1} = 2 u^i - u^{i-1} + dt^2 (A u^i + f^i) / rho,   u^0 = u^-1 = 0,
 * with f^i = signal[shot, i] * map in component src_comp, and records u^{i+1}
 * as frame i / stride when i % stride == 0 (Inversion_adam.py:299-301).
 * If `states` is non-NULL it receives u^0..u^nt for every shot, laid out
 * [n][shot][comp][cell], which is what oracle_adjoint consumes. */
int FN(oracle_forward)(const OracleProblem* p, const REAL* C, const REAL* D,
                       const REAL* src_signal, const REAL* src_map, const int32_t* src_origin,
                       const int32_t* rec_idx, REAL rho, REAL* out_ux, REAL* out_uy,
                       REAL* states) {
  int rc = oracle_check(p);
  if (rc) return rc;
  {
    const int nx = p->nx, ny = p->ny, nt = p->nt, S = p->nshots;
    const size_t N = (size_t)nx * ny;
    const int nt_out = (nt + p->stride - 1) / p->stride;
    const REAL dt2 = (REAL)(p->dt * p->dt);
    REAL* buf = (REAL*)calloc(7 * N, sizeof(REAL));
    REAL *ux1 = buf, *uy1 = buf + N, *ux2 = buf + 2 * N, *uy2 = buf + 3 * N;
    REAL *Lx = buf + 4 * N, *Ly = buf + 5 * N, *f = buf + 6 * N;
    int s, i;
    if (!buf) return ORACLE_ERR_ALLOC;
    for (s = 0; s < S; ++s) {
      memset(buf, 0, 7 * N * sizeof(REAL));
      if (states) {
        memset(states + ((size_t)0 * S + s) * 2 * N, 0, 2 * N * sizeof(REAL));
      }
      for (i = 0; i < nt; ++i) {
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
            f[(size_t)xi * ny + yj] =
                amp * src_map[((size_t)s * p->src_bx + a) * p->src_by + b];
          }
        FN(apply_operator)(p, C, D, ux1, uy1, p->src_comp == 0 ? f : NULL,
                           p->src_comp == 1 ? f : NULL, rho, Lx, Ly);
#pragma omp parallel for schedule(static)
        for (cc = 0; cc < (long)N; ++cc) {
          /* Inversion_adam.py:286-287, evaluated ((2u) - u') + dt^2 L */
          const REAL nxv = ((REAL)2 * ux1[cc] - ux2[cc]) + dt2 * Lx[cc];
          const REAL nyv = ((REAL)2 * uy1[cc] - uy2[cc]) + dt2 * Ly[cc];
          ux2[cc] = nxv; /* u^{i-1} slot now holds u^{i+1} */
          uy2[cc] = nyv;
        }
        { REAL* t = ux1; ux1 = ux2; ux2 = t; t = uy1; uy1 = uy2; uy2 = t; }
        if (states) {
          REAL* dst = states + ((size_t)(i + 1) * S + s) * 2 * N;
          memcpy(dst, ux1, N * sizeof(REAL));
          memcpy(dst + N, uy1, N * sizeof(REAL));
        }
        if (i % p->stride == 0) {
          const int fr = i / p->stride;
          if (p->record == ORACLE_RECORD_FIELDS) {
            memcpy(out_ux + ((size_t)s * nt_out + fr) * N, ux1, N * sizeof(REAL));
            memcpy(out_uy + ((size_t)s * nt_out + fr) * N, uy1, N * sizeof(REAL));
          } else {
            int r;
            for (r = 0; r < p->nrec; ++r) {
              const int32_t c = rec_idx[(size_t)s * p->nrec + r];
              out_ux[((size_t)s * nt_out + fr) * p->nrec + r] = ux1[c];
              out_uy[((size_t)s * nt_out + fr) * p->nrec + r] = uy1[c];
            }
          }
        }
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

/* Exact discrete adjoint of oracle_forward (what loss.backward() computes at
 * Inversion_adam.py:447 / Damage_inversion/Inversion_adam.py:511).
 * With kappa = dt^2 / rho and lam^m = dL/du^m:
 *   lam^m = g^m + 2 lam^{m+1} - lam^{m+2} + kappa A^T lam^{m+1},  m = nt..1
 *   dL/dC = kappa sum_{n} lam^{n+1} . d(A u^n)/dC
 * g^m is the output gradient of the frame that recorded u^m.  Gradients are
 * accumulated in double.  Outputs:
 *   SCALAR: grad_C[6]   (C11, C22, C12, C16, C26, C66)
 *   FIELDS: grad_C[6*N] per-cell planes
 *   DFIELD: grad_D[N]   dL/dD = -sum_t C0_t dL/dC_t(x); grad_C may be NULL */
int FN(oracle_adjoint)(const OracleProblem* p, const REAL* C, const REAL* D, REAL rho,
                       const int32_t* rec_idx, const REAL* states, const REAL* g_ux,
                       const REAL* g_uy, double* grad_C, double* grad_D) {
  int rc = oracle_check(p);
  if (rc) return rc;
  {
    const int nx = p->nx, ny = p->ny, nt = p->nt, S = p->nshots;
    const size_t N = (size_t)nx * ny;
    const int nt_out = (nt + p->stride - 1) / p->stride;
    const REAL dt2 = (REAL)(p->dt * p->dt);
    const REAL kappa = dt2 / rho;
    const REAL hinv2 = (REAL)(1.0 / (p->h * p->h));
    const REAL w1 = hinv2, w2 = hinv2 * (REAL)-2, wq = hinv2 * (REAL)0.25;
    const int percell = (p->mode != ORACLE_MODE_SCALAR);
    REAL* buf = (REAL*)calloc(14 * N, sizeof(REAL));
    double* acc = (double*)calloc(percell ? 6 * N : 6, sizeof(double));
    REAL *l1x = buf, *l1y = buf + N, *l2x = buf + 2 * N, *l2y = buf + 3 * N;
    REAL *tx = buf + 4 * N, *ty = buf + 5 * N, *P = buf + 6 * N;
    int s, m, t;
    if (!buf || !acc) { free(buf); free(acc); return ORACLE_ERR_ALLOC; }
    for (s = 0; s < S; ++s) {
      memset(buf, 0, 6 * N * sizeof(REAL));
      for (m = nt; m >= 1; --m) {
        long cc;
        /* imaging term n = m: lam^{m+1} . d(A u^m)/dC (zero when m == nt) */
        if (m <= nt - 1) {
          const REAL* ux = states + ((size_t)m * S + s) * 2 * N;
          const REAL* uy = ux + N;
          double sums[6] = {0, 0, 0, 0, 0, 0};
          for (cc = 0; cc < (long)N; ++cc) {
            const int i = (int)(cc / ny), j = (int)(cc % ny);
            const double a = l1x[cc], b = l1y[cc];
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
              for (t = 0; t < 6; ++t) acc[(size_t)t * N + cc] += (double)kappa * g[t];
            } else {
              for (t = 0; t < 6; ++t) sums[t] += g[t];
            }
          }
          if (!percell)
            for (t = 0; t < 6; ++t) acc[t] += (double)kappa * sums[t];
        }
        /* lam^m = 2 lam^{m+1} - lam^{m+2} + kappa A^T lam^{m+1} + g^m */
        FN(apply_transpose)(p, C, D, l1x, l1y, P, tx, ty);
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
        { REAL* q = l1x; l1x = l2x; l2x = q; q = l1y; l1y = l2y; l2y = q; }
      }
    }
    if (!percell) {
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
        if (grad_C) {
          /* dL/dC0_t = sum_x (1 - D(x)) dL/dC_t(x) */
          for (t = 0; t < 6; ++t) grad_C[t] += (1.0 - (double)D[c]) * acc[(size_t)t * N + c];
        }
      }
    }
    free(buf);
    free(acc);
  }
  return 0;
}

#undef AT
