/*
 * CPU oracle for heatsim2's ADI Crank-Nicolson timestep.  TEST INFRASTRUCTURE ONLY: it is the checker that
 * tests/, __graft_entry__.smoke() and bench.py's cpu_baseline leg compare the CUDA path against; the
 * product never links or calls it.
 *
 * It restates the reference algorithm in the reference's own matrix form (not the scaled delta form the
 * CUDA kernels use), so a mistake in the GPU formulation cannot be shared by the oracle:
 *
 *   setup      crank_nicolson.pyx:272-491   per-voxel heat balance: neighbour-k fallback (:298-338),
 *                                          face fluxes of the four built-in boundary classes, time term (:378),
 *                                          fixed-temperature rows (:473-486)
 *              alternatingdirection_c_pyx.pyx:475-493  Douglas stage split x -> y -> z (crank_subst_in_groups)
 *              alternatingdirection_c.c:102-199        scatter into A (tridiagonal), B, C_j (sparse), D,
 *                                                      rows numbered in the stage's permuted order (:114)
 *              tridiag.pyx:9-43                        tridiaglu, once per stage
 *   step       alternatingdirection_c_pyx.pyx:387-416  rhs = B*T + sum_j C_j*T*_j + D*Q, tridiagsolve,
 *                                                      un-permute; returns the last stage
 *              tridiag.pyx:46-69                       tridiagsolve
 *
 * Boundary classes (per-face conductance G, W/m^3/K, the coefficient of T_nbr - T_p in the heat balance):
 *   insulating                0                                         boundary_insulating.py:2-34
 *   conducting                0.5*(k_lo+k_hi) * (1/d) * (1/d)           boundary_conducting.py:18-25
 *   conducting_anisotropic    0.5*(K_lo[a][a]+K_hi[a][a]) * (1/d)*(1/d) boundary_conducting_anisotropic.py:24,44,65
 *   thininsulatinglayer(h)    h * (1/d)                                 boundary_thininsulatinglayer.py:19-23
 * with the heat-balance division by the cell size of crank_nicolson.pyx:359-362.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

enum { OR_MAT_COMPUTE = 0, OR_MAT_FIXED = 1 };
enum { OR_BND_INSULATING = 0, OR_BND_CONDUCTING = 1, OR_BND_ANISOTROPIC = 2, OR_BND_THIN = 3 };

/* error codes */
#define OR_OK 0
#define OR_ERR_EXTERIOR (-2)   /* non-insulating exterior face: alternatingdirection_c.c:158-163 exits */
#define OR_ERR_KTYPE (-3)      /* scalar class on matrix k or the reverse (expression.py:303-306) */
#define OR_ERR_ALLOC (-4)
#define OR_ERR_ARG (-5)

/* fixed-width rows (at most 7 B entries and 3 C entries per row), columns ascending, duplicates summed:
   the same row contents scipy's coo_matrix(...).tocsr() holds (alternatingdirection_c_pyx.pyx:251,:269) */
typedef struct {
  int width;
  int32_t *col;
  double *val;
  uint8_t *cnt;
} ell_t;

typedef struct {
  int64_t nz, ny, nx, n;
  double *A[3];
  double *L[3];
  double *U[3];
  ell_t B[3];
  ell_t C[3][2];
  double *D[3];
  /* scratch for one step */
  double *perm_in, *rhs, *sol, *stage[3];
} oracle_adi;

/* stage s uses permuteorder (0,1,2), (2,0,1), (1,2,0) (alternatingdirection_c_pyx.pyx:426-432) */
static inline int64_t prow(const oracle_adi *o, int s, int64_t k, int64_t j, int64_t i) {
  if (s == 0) return (k * o->ny + j) * o->nx + i;         /* permuted shape (nz,ny,nx) */
  if (s == 1) return (i * o->nz + k) * o->ny + j;         /* permuted shape (nx,nz,ny) */
  return (j * o->nx + i) * o->nz + k;                     /* permuted shape (ny,nx,nz) */
}

typedef struct {
  int32_t col;
  double val;
} entry_t;

static int cmp_entry(const void *a, const void *b) {
  int32_t ca = ((const entry_t *)a)->col, cb = ((const entry_t *)b)->col;
  return (ca > cb) - (ca < cb);
}

static void ell_row(ell_t *m, int64_t row, entry_t *e, int ne) {
  if (ne > 1) qsort(e, (size_t)ne, sizeof(entry_t), cmp_entry);
  int32_t *col = m->col + row * m->width;
  double *val = m->val + row * m->width;
  int pos = 0;
  for (int c = 0; c < ne; ++c) {
    if (pos > 0 && e[c].col == col[pos - 1]) {
      val[pos - 1] += e[c].val;
    } else {
      col[pos] = e[c].col;
      val[pos] = e[c].val;
      ++pos;
    }
  }
  m->cnt[row] = (uint8_t)pos;
}

static int ell_alloc(ell_t *m, int64_t n, int width) {
  m->width = width;
  m->col = (int32_t *)calloc((size_t)(n * width), sizeof(int32_t));
  m->val = (double *)calloc((size_t)(n * width), sizeof(double));
  m->cnt = (uint8_t *)calloc((size_t)n, 1);
  return (m->col && m->val && m->cnt) ? OR_OK : OR_ERR_ALLOC;
}

static void ell_free(ell_t *m) {
  free(m->col);
  free(m->val);
  free(m->cnt);
  memset(m, 0, sizeof(*m));
}

/* y (+)= M x, each row summed in column order like scipy's csr_matvec */
static void ell_matvec(const ell_t *m, int64_t n, const double *x, double *y, int accumulate) {
  for (int64_t r = 0; r < n; ++r) {
    const int32_t *col = m->col + r * m->width;
    const double *val = m->val + r * m->width;
    double acc = 0.0;
    for (int c = 0; c < m->cnt[r]; ++c) acc += val[c] * x[col[c]];
    y[r] = accumulate ? y[r] + acc : acc;
  }
}

void oracle_free(oracle_adi *o) {
  if (!o) return;
  for (int s = 0; s < 3; ++s) {
    free(o->A[s]);
    free(o->L[s]);
    free(o->U[s]);
    free(o->D[s]);
    free(o->stage[s]);
    ell_free(&o->B[s]);
    for (int c = 0; c < 2; ++c) ell_free(&o->C[s][c]);
  }
  free(o->perm_in);
  free(o->rhs);
  free(o->sol);
  free(o);
}

/* tridiag.pyx:9-43 */
void oracle_tridiaglu(int64_t n, const double *A, double *L, double *U) {
  memset(L, 0, (size_t)n * 3 * sizeof(double));
  memcpy(U, A, (size_t)n * 3 * sizeof(double));
  for (int64_t row = 0; row < n; ++row) {
    L[row * 3 + 1] = U[row * 3 + 1];
    U[row * 3 + 2] /= U[row * 3 + 1];
    U[row * 3 + 1] = 1.0;
    if (row < n - 1) {
      double coefficient = U[(row + 1) * 3 + 0];
      U[(row + 1) * 3 + 0] = 0.0;
      U[(row + 1) * 3 + 1] -= U[row * 3 + 2] * coefficient;
      L[(row + 1) * 3 + 0] = coefficient;
    }
  }
}

/* tridiag.pyx:46-69 */
void oracle_tridiagsolve(int64_t n, const double *L, const double *U, const double *b, double *x) {
  if (n <= 0) return;
  x[0] = b[0] / L[1];
  for (int64_t row = 1; row < n; ++row) x[row] = (b[row] - L[row * 3 + 0] * x[row - 1]) / L[row * 3 + 1];
  for (int64_t row = n - 2; row >= 0; --row) x[row] = x[row] - U[row * 3 + 2] * x[row + 1];
}

/*
 * Per-face conductance for the class of one face, seen from a compute voxel: k_lo / k_hi are the
 * conductivities on the low / high side after the neighbour-k fallback.  kmat[] holds scalar k in [0] when
 * is_matrix is 0, or the (z,y,x) diagonal of a 3x3 K when is_matrix is 1.
 */
static int face_G(int bkind, double h, int axis, double inv_d, int lo_matrix, const double *klo, int hi_matrix,
                  const double *khi, double *G) {
  switch (bkind) {
    case OR_BND_INSULATING:
      *G = 0.0;
      return OR_OK;
    case OR_BND_CONDUCTING:
      if (lo_matrix || hi_matrix) return OR_ERR_KTYPE;
      *G = (klo[0] + khi[0]) * 0.5 * inv_d * inv_d;
      return OR_OK;
    case OR_BND_ANISOTROPIC:
      if (!lo_matrix || !hi_matrix) return OR_ERR_KTYPE;
      *G = (klo[axis] + khi[axis]) * 0.5 * inv_d * inv_d;
      return OR_OK;
    case OR_BND_THIN:
      *G = h * inv_d;
      return OR_OK;
  }
  return OR_ERR_ARG;
}

/*
 * material_kind[m]  OR_MAT_COMPUTE / OR_MAT_FIXED
 * material_k[m*3+a] scalar k in [m*3] (is_matrix 0) or diagonal of K in z,y,x order (is_matrix 1)
 * material_rho_c_over_dt[m]  rho*c*(1/dt)
 * boundary_kind[b], boundary_h[b]
 */
int oracle_setup(int64_t nz, int64_t ny, int64_t nx, double dz, double dy, double dx, const uint8_t *material,
                 const uint8_t *bz, const uint8_t *by, const uint8_t *bx, int nmat, const int32_t *material_kind,
                 const int32_t *material_is_matrix, const double *material_k, const double *material_M, int nbnd,
                 const int32_t *boundary_kind, const double *boundary_h, oracle_adi **out) {
  *out = NULL;
  if (nz < 1 || ny < 1 || nx < 1) return OR_ERR_ARG;
  oracle_adi *o = (oracle_adi *)calloc(1, sizeof(oracle_adi));
  if (!o) return OR_ERR_ALLOC;
  o->nz = nz;
  o->ny = ny;
  o->nx = nx;
  const int64_t n = nz * ny * nx;
  o->n = n;
  int rc = OR_OK;
  for (int s = 0; s < 3; ++s) {
    o->A[s] = (double *)calloc((size_t)n * 3, sizeof(double));
    o->L[s] = (double *)calloc((size_t)n * 3, sizeof(double));
    o->U[s] = (double *)calloc((size_t)n * 3, sizeof(double));
    o->D[s] = (double *)calloc((size_t)n, sizeof(double));
    o->stage[s] = (double *)calloc((size_t)n, sizeof(double));
    if (!o->A[s] || !o->L[s] || !o->U[s] || !o->D[s] || !o->stage[s]) rc = OR_ERR_ALLOC;
    if (rc == OR_OK) rc = ell_alloc(&o->B[s], n, 7);
    for (int c = 0; c < s && rc == OR_OK; ++c) rc = ell_alloc(&o->C[s][c], n, 3);
  }
  o->perm_in = (double *)malloc((size_t)n * sizeof(double));
  o->rhs = (double *)malloc((size_t)n * sizeof(double));
  o->sol = (double *)malloc((size_t)n * sizeof(double));
  if (!o->perm_in || !o->rhs || !o->sol) rc = OR_ERR_ALLOC;
  if (rc != OR_OK) {
    oracle_free(o);
    return rc;
  }
  const double inv_d[3] = {1.0 / dz, 1.0 / dy, 1.0 / dx};
  /* stage of each axis (z,y,x) and axis of each stage: x first, then y, then z */
  const int stage_of_axis[3] = {2, 1, 0};
  const int64_t sz[3] = {nz, ny, nx};

  for (int64_t k = 0; k < nz && rc == OR_OK; ++k)
    for (int64_t j = 0; j < ny && rc == OR_OK; ++j)
      for (int64_t i = 0; i < nx && rc == OR_OK; ++i) {
        const int64_t p = (k * ny + j) * nx + i;
        const int m = material[p];
        if (m >= nmat) {
          rc = OR_ERR_ARG;
          break;
        }
        const int64_t idx[3] = {k, j, i};
        if (material_kind[m] != OR_MAT_COMPUTE) {
          /* fixed temperature: identity row in every stage, D = 0 (crank_nicolson.pyx:473-486) */
          for (int s = 0; s < 3; ++s) {
            const int64_t r = prow(o, s, k, j, i);
            o->A[s][r * 3 + 1] = 1.0;
            entry_t e = {(int32_t)r, 1.0};
            ell_row(&o->B[s], r, &e, 1);
          }
          continue;
        }
        const double *kown = material_k + 3 * m;
        const int own_matrix = material_is_matrix[m];
        double Glo[3], Ghi[3];
        for (int a = 0; a < 3 && rc == OR_OK; ++a) {
          /* neighbour k: the neighbour's if it is inside the grid and computed, else the voxel's own
             (crank_nicolson.pyx:298-338) */
          const double *knb[2];
          int nb_matrix[2];
          int exterior[2];
          for (int side = 0; side < 2; ++side) {
            int64_t q[3] = {idx[0], idx[1], idx[2]};
            q[a] += side ? 1 : -1;
            exterior[side] = (q[a] < 0 || q[a] >= sz[a]);
            knb[side] = kown;
            nb_matrix[side] = own_matrix;
            if (!exterior[side]) {
              const int mq = material[(q[0] * ny + q[1]) * nx + q[2]];
              if (mq < nmat && material_kind[mq] == OR_MAT_COMPUTE) {
                knb[side] = material_k + 3 * mq;
                nb_matrix[side] = material_is_matrix[mq];
              }
            }
          }
          /* face class indices: the low face of voxel idx along a has index idx[a] */
          uint8_t blo, bhi;
          if (a == 0) {
            blo = bz[(k * ny + j) * nx + i];
            bhi = bz[((k + 1) * ny + j) * nx + i];
          } else if (a == 1) {
            blo = by[(k * (ny + 1) + j) * nx + i];
            bhi = by[(k * (ny + 1) + j + 1) * nx + i];
          } else {
            blo = bx[(k * ny + j) * (nx + 1) + i];
            bhi = bx[(k * ny + j) * (nx + 1) + i + 1];
          }
          if (blo >= nbnd || bhi >= nbnd) {
            rc = OR_ERR_ARG;
            break;
          }
          rc = face_G(boundary_kind[blo], boundary_h[blo], a, inv_d[a], nb_matrix[0], knb[0], own_matrix, kown,
                      &Glo[a]);
          if (rc == OR_OK)
            rc = face_G(boundary_kind[bhi], boundary_h[bhi], a, inv_d[a], own_matrix, kown, nb_matrix[1], knb[1],
                        &Ghi[a]);
          if (rc == OR_OK && ((exterior[0] && Glo[a] != 0.0) || (exterior[1] && Ghi[a] != 0.0)))
            rc = OR_ERR_EXTERIOR;
        }
        if (rc != OR_OK) break;
        const double M = material_M[m];
        for (int s = 0; s < 3; ++s) {
          const int64_t r = prow(o, s, k, j, i);
          entry_t eb[16];
          int nb = 0;
          entry_t ec[2][8];
          int ncc[2] = {0, 0};
          double center_B = M;   /* time term -(T+ - T-)*rho*c/dt: +M on T- (B) */
          double diag_A = M;     /* and -(-M) on the solved T+ (A = minus coefficient) */
          for (int a = 0; a < 3; ++a) {
            const int sa = stage_of_axis[a];
            const double w = (sa <= s) ? 0.5 : 1.0; /* Crank-Nicolson halves once the axis has been solved */
            int64_t qlo[3] = {idx[0], idx[1], idx[2]}, qhi[3] = {idx[0], idx[1], idx[2]};
            qlo[a] -= 1;
            qhi[a] += 1;
            if (Glo[a] != 0.0) {
              eb[nb++] = (entry_t){(int32_t)prow(o, s, qlo[0], qlo[1], qlo[2]), w * Glo[a]};
              center_B -= w * Glo[a];
              if (sa == s) {
                o->A[s][r * 3 + 0] = -(0.5 * Glo[a]);
                diag_A += 0.5 * Glo[a];
              } else if (sa < s) {
                ec[sa][ncc[sa]++] = (entry_t){(int32_t)prow(o, s, qlo[0], qlo[1], qlo[2]), 0.5 * Glo[a]};
                ec[sa][ncc[sa]++] = (entry_t){(int32_t)r, -(0.5 * Glo[a])};
              }
            }
            if (Ghi[a] != 0.0) {
              eb[nb++] = (entry_t){(int32_t)prow(o, s, qhi[0], qhi[1], qhi[2]), w * Ghi[a]};
              center_B -= w * Ghi[a];
              if (sa == s) {
                o->A[s][r * 3 + 2] = -(0.5 * Ghi[a]);
                diag_A += 0.5 * Ghi[a];
              } else if (sa < s) {
                ec[sa][ncc[sa]++] = (entry_t){(int32_t)prow(o, s, qhi[0], qhi[1], qhi[2]), 0.5 * Ghi[a]};
                ec[sa][ncc[sa]++] = (entry_t){(int32_t)r, -(0.5 * Ghi[a])};
              }
            }
          }
          eb[nb++] = (entry_t){(int32_t)r, center_B};
          o->A[s][r * 3 + 1] = diag_A;
          o->D[s][r] = 1.0; /* coefficient of volumetric_source (alternatingdirection_c.c:119-121) */
          ell_row(&o->B[s], r, eb, nb);
          for (int c = 0; c < s; ++c) ell_row(&o->C[s][c], r, ec[c], ncc[c]);
        }
      }
  if (rc != OR_OK) {
    oracle_free(o);
    return rc;
  }
  for (int s = 0; s < 3; ++s) oracle_tridiaglu(n, o->A[s], o->L[s], o->U[s]);
  *out = o;
  return OR_OK;
}

/* permute a natural-order (nz,ny,nx) field into stage s's row order: Tarray.transpose(perm).reshape(n) */
static void permute_in(const oracle_adi *o, int s, const double *src, double *dst) {
  for (int64_t k = 0; k < o->nz; ++k)
    for (int64_t j = 0; j < o->ny; ++j)
      for (int64_t i = 0; i < o->nx; ++i) dst[prow(o, s, k, j, i)] = src[(k * o->ny + j) * o->nx + i];
}

static void permute_out(const oracle_adi *o, int s, const double *src, double *dst) {
  for (int64_t k = 0; k < o->nz; ++k)
    for (int64_t j = 0; j < o->ny; ++j)
      for (int64_t i = 0; i < o->nx; ++i) dst[(k * o->ny + j) * o->nx + i] = src[prow(o, s, k, j, i)];
}

/* One timestep (alternatingdirection_c_pyx.pyx:387-416).  Q is the evaluated source field (natural order,
   W/m^3; pyx:294-386 is evaluated by the caller).  T_out may alias T_in. */
int oracle_step(oracle_adi *o, const double *T_in, const double *Q, double *T_out) {
  const int64_t n = o->n;
  for (int s = 0; s < 3; ++s) {
    permute_in(o, s, T_in, o->perm_in);
    ell_matvec(&o->B[s], n, o->perm_in, o->rhs, 0);
    for (int c = 0; c < s; ++c) {
      permute_in(o, s, o->stage[c], o->perm_in);
      ell_matvec(&o->C[s][c], n, o->perm_in, o->rhs, 1);
    }
    permute_in(o, s, Q, o->perm_in);
    for (int64_t r = 0; r < n; ++r) o->rhs[r] += o->D[s][r] * o->perm_in[r];
    oracle_tridiagsolve(n, o->L[s], o->U[s], o->rhs, o->sol);
    permute_out(o, s, o->sol, o->stage[s]);
  }
  memcpy(T_out, o->stage[2], (size_t)n * sizeof(double));
  return OR_OK;
}

int64_t oracle_voxels(const oracle_adi *o) { return o->n; }

/* Export stage s's matrices for tests: A (n x 3), D (n), and B / C rows as (row, col, val) triples.
   Returns the number of triples written for the requested matrix (which = 0 for B, 1 + c for C_c). */
int64_t oracle_export(const oracle_adi *o, int s, int which, double *A, double *D, int64_t *rows, int64_t *cols,
                      double *vals) {
  const int64_t n = o->n;
  if (A) memcpy(A, o->A[s], (size_t)n * 3 * sizeof(double));
  if (D) memcpy(D, o->D[s], (size_t)n * sizeof(double));
  const ell_t *m = which == 0 ? &o->B[s] : &o->C[s][which - 1];
  int64_t cnt = 0;
  for (int64_t r = 0; r < n; ++r)
    for (int c = 0; c < m->cnt[r]; ++c) {
      if (rows) {
        rows[cnt] = r;
        cols[cnt] = m->col[r * m->width + c];
        vals[cnt] = m->val[r * m->width + c];
      }
      ++cnt;
    }
  return cnt;
}
