/*
 * Body of the FEM generator oracle (see fem_oracle.c), included once per
 * precision.  TEST INFRASTRUCTURE ONLY.
 *
 * load:   (nx * ny) nodal Gaussian, node id j*nx + i (FEM_generate_data.py:308, `.T.flatten()`)
 * signal: (nt) Ricker time factors (:461-463)
 * Cf:     NULL (p->C everywhere) or 6 planes (nx, ny) of per-node constants
 *         (the damaged-plate generator, Damage_inversion/FEM_generate_data.py)
 * frames_x/y: (nt_out, nx, ny), nt_out = ceil(nt / stride)
 */
int FN(oracle_fem_forward)(const OracleFemProblem* p, const REAL* load, const REAL* signal,
                           const REAL* Cf, REAL* frames_x, REAL* frames_y) {
  if (!p || p->nx < 2 || p->ny < 2 || p->nt < 1 || p->stride < 1) return FEM_ERR_INVALID;
  const int nx = p->nx, ny = p->ny, nt = p->nt;
  const size_t nn = (size_t)nx * ny;
  const size_t ne = (size_t)2 * (nx - 1) * (ny - 1);
  const int nt_out = (nt + p->stride - 1) / p->stride;
  int32_t* el = (int32_t*)malloc(ne * 3 * sizeof(int32_t));
  REAL* M = (REAL*)calloc(nn, sizeof(REAL));
  REAL* ux = (REAL*)calloc(3 * nn, sizeof(REAL));
  REAL* uy = (REAL*)calloc(3 * nn, sizeof(REAL));
  REAL* fx = (REAL*)malloc(nn * sizeof(REAL));
  REAL* fy = (REAL*)malloc(nn * sizeof(REAL));
  REAL* bx = (REAL*)malloc(ne * 3 * sizeof(REAL)); /* dN/dx per element node */
  REAL* by = (REAL*)malloc(ne * 3 * sizeof(REAL));
  REAL* fac = (REAL*)malloc(ne * sizeof(REAL));     /* |det J| per element */
  REAL* ce = (REAL*)malloc(ne * 6 * sizeof(REAL));  /* constants per element */
  char* bnd = (char*)calloc(nn, 1);
  if (!el || !M || !ux || !uy || !fx || !fy || !bx || !by || !fac || !bnd || !ce) {
    free(el); free(M); free(ux); free(uy); free(fx); free(fy); free(bx); free(by); free(fac); free(bnd);
    free(ce);
    return FEM_ERR_ALLOC;
  }
  /* mesh (:150-168) */
  size_t e = 0;
  for (int j = 0; j < ny - 1; ++j)
    for (int i = 0; i < nx - 1; ++i) {
      const int32_t n0 = j * nx + i, n1 = j * nx + i + 1, n2 = (j + 1) * nx + i + 1, n3 = (j + 1) * nx + i;
      const int32_t* t = ((i + j) % 2 == 0) ? (int32_t[6]){n0, n1, n2, n0, n2, n3}
                                            : (int32_t[6]){n0, n1, n3, n1, n2, n3};
      memcpy(el + 3 * e, t, 6 * sizeof(int32_t));
      e += 2;
    }
  for (int i = 0; i < nx; ++i) { bnd[i] = 1; bnd[(size_t)(ny - 1) * nx + i] = 1; }
  for (int j = 0; j < ny; ++j) { bnd[(size_t)j * nx] = 1; bnd[(size_t)j * nx + nx - 1] = 1; }
  /* lumped mass (:334-340) */
  const REAL mnode = (REAL)(p->rho * (p->dx * p->dy / 2.0) / 3.0);
  for (e = 0; e < ne; ++e)
    for (int a = 0; a < 3; ++a) M[el[3 * e + a]] += mnode;
  /* element geometry (:365-384): coordinates x_i = -Lx/2 + i dx; J and its
   * inverse in double, then rounded to REAL as the reference moves them to
   * float32 tensors */
  for (e = 0; e < ne; ++e) {
    double xc[3], yc[3];
    for (int a = 0; a < 3; ++a) {
      const int32_t n = el[3 * e + a];
      xc[a] = (n % nx) * p->dx;
      yc[a] = (n / nx) * p->dy;
    }
    const double J00 = xc[1] - xc[0], J01 = xc[2] - xc[0], J10 = yc[1] - yc[0], J11 = yc[2] - yc[0];
    const double det = J00 * J11 - J01 * J10;
    const double i00 = J11 / det, i01 = -J01 / det, i10 = -J10 / det, i11 = J00 / det;
    const REAL r00 = (REAL)i00, r01 = (REAL)i01, r10 = (REAL)i10, r11 = (REAL)i11;
    static const double dxi[3] = {-1.0, 1.0, 0.0}, deta[3] = {-1.0, 0.0, 1.0};
    for (int a = 0; a < 3; ++a) {
      bx[3 * e + a] = r00 * (REAL)dxi[a] + r10 * (REAL)deta[a];
      by[3 * e + a] = r01 * (REAL)dxi[a] + r11 * (REAL)deta[a];
    }
    fac[e] = (REAL)fabs(det);
    /* constants: uniform, or those of the grid node nearest the element's
     * centroid (argmin |x - mean(x)|, argmin |y - mean(y)|;
     * Damage_inversion/FEM_generate_data.py:1002-1017) */
    if (Cf == NULL) {
      for (int c = 0; c < 6; ++c) ce[6 * e + c] = (REAL)p->C[c];
    } else {
      const double mx = (xc[0] + xc[1] + xc[2]) / 3.0, my = (yc[0] + yc[1] + yc[2]) / 3.0;
      int bi = 0, bj = 0;
      for (int i = 1; i < nx; ++i)
        if (fabs(i * p->dx - mx) < fabs(bi * p->dx - mx)) bi = i;
      for (int j = 1; j < ny; ++j)
        if (fabs(j * p->dy - my) < fabs(bj * p->dy - my)) bj = j;
      for (int c = 0; c < 6; ++c) ce[6 * e + c] = Cf[(size_t)c * nn + (size_t)bi * ny + bj];
    }
  }
  const REAL w = (REAL)(1.0 / 6.0);
  const REAL dt2 = (REAL)(p->dt * p->dt);
  const REAL rho_inv = (REAL)(1.0 / p->rho);
  const REAL sc = (REAL)p->out_scale;
  /* frame 0 = u^0 = 0 */
  for (size_t k = 0; k < nn; ++k) { frames_x[k] = 0; frames_y[k] = 0; }
  /* levels: slot (n % 3) holds u^n */
  for (int n = 1; n < nt - 1; ++n) {
    const REAL* cx = ux + (size_t)(n % 3) * nn;
    const REAL* cy = uy + (size_t)(n % 3) * nn;
    const REAL* px = ux + (size_t)((n + 2) % 3) * nn;
    const REAL* py = uy + (size_t)((n + 2) % 3) * nn;
    REAL* ox = ux + (size_t)((n + 1) % 3) * nn;
    REAL* oy = uy + (size_t)((n + 1) % 3) * nn;
    memset(fx, 0, nn * sizeof(REAL));
    memset(fy, 0, nn * sizeof(REAL));
    for (int gp = 0; gp < 3; ++gp) { /* three Gauss points, identical B (:420-455) */
      for (e = 0; e < ne; ++e) {
        const int32_t* t = el + 3 * e;
        const REAL* gx = bx + 3 * e;
        const REAL* gy = by + 3 * e;
        REAL exx = 0, eyy = 0, gxy = 0;
        for (int a = 0; a < 3; ++a) {
          exx += gx[a] * cx[t[a]];
          eyy += gy[a] * cy[t[a]];
          gxy += gy[a] * cx[t[a]] + gx[a] * cy[t[a]];
        }
        const REAL* k6 = ce + 6 * e;
        const REAL C11 = k6[0], C22 = k6[1], C12 = k6[2], C16 = k6[3], C26 = k6[4], C66 = k6[5];
        const REAL sxx = C11 * exx + C12 * eyy + C16 * gxy;
        const REAL syy = C12 * exx + C22 * eyy + C26 * gxy;
        const REAL txy = C16 * exx + C26 * eyy + C66 * gxy;
        const REAL f = fac[e] * w;
        for (int a = 0; a < 3; ++a) {
          fx[t[a]] += f * (gx[a] * sxx + gy[a] * txy);
          fy[t[a]] += f * (gy[a] * syy + gx[a] * txy);
        }
      }
    }
    const REAL tf = signal[n];
    for (size_t k = 0; k < nn; ++k) {
      const REAL fext = (tf * load[k] * rho_inv) * M[k];
      REAL vx = 2 * cx[k] - px[k] - dt2 * fx[k] / M[k];
      REAL vy = 2 * cy[k] - py[k] + dt2 * (fext - fy[k]) / M[k];
      if (bnd[k]) { vx = 0; vy = 0; }
      ox[k] = vx;
      oy[k] = vy;
    }
    if ((n + 1) % p->stride == 0) {
      const size_t f = (size_t)((n + 1) / p->stride) * nn;
      for (int j = 0; j < ny; ++j)
        for (int i = 0; i < nx; ++i) {
          frames_x[f + (size_t)i * ny + j] = sc * ox[(size_t)j * nx + i];
          frames_y[f + (size_t)i * ny + j] = sc * oy[(size_t)j * nx + i];
        }
    }
  }
  /* frames of levels never computed (nt < 3 leaves u^1 = 0) */
  for (int k = 1; k < nt_out; ++k) {
    const int lev = k * p->stride;
    if (lev <= 1) {
      memset(frames_x + (size_t)k * nn, 0, nn * sizeof(REAL));
      memset(frames_y + (size_t)k * nn, 0, nn * sizeof(REAL));
    }
  }
  free(el); free(M); free(ux); free(uy); free(fx); free(fy); free(bx); free(by); free(fac); free(bnd);
  free(ce);
  return 0;
}
