/*
 * CPU baseline of the field step with the GPU's algorithm: matrix-free geometric
 * multigrid preconditioned CG in FP64, one trap per OpenMP thread.
 *
 * TEST/BENCH INFRASTRUCTURE ONLY (the timed "all host cores, same algorithm" CPU
 * baseline; its solutions are checked against the SuperLU oracle in the tests).
 *
 * One step of one trap solves ((1 + dt g) M + dt D K) u' = M u + F on the "right"
 * triangulation of [0, W] x [0, H] (the hslD bilinear form, fenics/hslD.ufl:31-49,
 * for an isotropic tensor; zero Dirichlet rows on the walls' nodes, their couplings
 * removed so the operator stays symmetric).  Levels coarsen each axis by taking every
 * other node and the last one (ragged last cell for odd counts) while it has at
 * least 4 cells; every level rediscretises the form on its own node positions.
 * Transfers: bilinear interpolation from the coarse nodes, restriction its
 * transpose.  V(2,2) cycle with Chebyshev-Jacobi smoothing on [lmax/5, lmax]
 * (lmax: Gershgorin bound of D^-1 A), dense Cholesky on the coarsest level.  The
 * outer CG runs to |b - A u| <= rtol |b| from the previous field.
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define MAXLEV 16

typedef struct {
  int nx, ny;     /* cells */
  double *xs, *ys; /* node positions (nx+1, ny+1) */
  double *st;     /* per node: c, e, w, n, s, ne, sw (7 doubles) */
  double *idg;    /* 1 / diagonal */
  double lmax;
  unsigned char* dir; /* Dirichlet node */
  double *x, *b, *r, *d, *t; /* work vectors */
  /* coarsest level: dense Cholesky factor (lower, row major) */
  double* chol;
  int nfree;
  int* freeidx;
} Level;

typedef struct {
  int nlev;
  Level L[MAXLEV];
  double alpha, beta;
} Hier;

static double now_s(void) {
  struct timespec ts;
  clock_gettime(CLOCK_MONOTONIC, &ts);
  return (double)ts.tv_sec + 1e-9 * (double)ts.tv_nsec;
}

static int coarse_count(int n) { return n >= 4 ? (n + 1) / 2 : n; }

static void coarse_positions(const double* f, int n, double* c, int nc) {
  if (nc == n) {
    memcpy(c, f, sizeof(double) * (size_t)(n + 1));
    return;
  }
  for (int J = 0; J < nc; ++J) c[J] = f[2 * J];
  c[nc] = f[n];
}

static int is_dir(unsigned walls, int i, int j, int nx, int ny) {
  return ((walls & 1u) && i == 0) || ((walls & 2u) && i == ny) || ((walls & 4u) && j == 0) ||
         ((walls & 8u) && j == nx);
}

/* rows of the operator alpha M + beta K on a tensor grid (right cut) */
static void build_level(Level* L, double alpha, double beta, unsigned walls) {
  const int nx = L->nx, ny = L->ny, P = nx + 1, n = P * (ny + 1);
  L->st = (double*)calloc((size_t)n * 7, sizeof(double));
  L->idg = (double*)calloc((size_t)n, sizeof(double));
  L->dir = (unsigned char*)calloc((size_t)n, 1);
  double lmax = 0.0;
  for (int i = 0; i <= ny; ++i)
    for (int j = 0; j <= nx; ++j) {
      const int k = j + i * P;
      double* s = L->st + 7 * (size_t)k;
      L->dir[k] = (unsigned char)is_dir(walls, i, j, nx, ny);
      if (L->dir[k]) {
        s[0] = 1.0;
        L->idg[k] = 1.0;
        continue;
      }
      const double hxl = j > 0 ? L->xs[j] - L->xs[j - 1] : 0.0;
      const double hxr = j < nx ? L->xs[j + 1] - L->xs[j] : 0.0;
      const double hyd = i > 0 ? L->ys[i] - L->ys[i - 1] : 0.0;
      const double hyu = i < ny ? L->ys[i + 1] - L->ys[i] : 0.0;
      const double sx = hxl + hxr, sy = hyd + hyu, hb = 0.5 * beta;
      const double a24 = alpha / 24.0, a12 = alpha / 12.0;
      const double ke = hxr > 0 ? hb * sy / hxr : 0.0, kw = hxl > 0 ? hb * sy / hxl : 0.0;
      const double kn = hyu > 0 ? hb * sx / hyu : 0.0, ks = hyd > 0 ? hb * sx / hyd : 0.0;
      s[1] = a24 * hxr * sy - ke;
      s[2] = a24 * hxl * sy - kw;
      s[3] = a24 * hyu * sx - kn;
      s[4] = a24 * hyd * sx - ks;
      s[5] = a12 * hxr * hyu;
      s[6] = a12 * hxl * hyd;
      s[0] = a12 * (2 * hxl * hyd + hxr * hyd + hxl * hyu + 2 * hxr * hyu) + ke + kw + kn + ks;
      /* couplings to Dirichlet neighbours removed */
      if (j < nx && is_dir(walls, i, j + 1, nx, ny)) s[1] = 0.0;
      if (j > 0 && is_dir(walls, i, j - 1, nx, ny)) s[2] = 0.0;
      if (i < ny && is_dir(walls, i + 1, j, nx, ny)) s[3] = 0.0;
      if (i > 0 && is_dir(walls, i - 1, j, nx, ny)) s[4] = 0.0;
      if (i < ny && j < nx && is_dir(walls, i + 1, j + 1, nx, ny)) s[5] = 0.0;
      if (i > 0 && j > 0 && is_dir(walls, i - 1, j - 1, nx, ny)) s[6] = 0.0;
      L->idg[k] = 1.0 / s[0];
      const double row = fabs(s[1]) + fabs(s[2]) + fabs(s[3]) + fabs(s[4]) + fabs(s[5]) +
                         fabs(s[6]);
      const double g = 1.0 + row / s[0];
      if (g > lmax) lmax = g;
    }
  L->lmax = lmax;
  L->x = (double*)calloc((size_t)n, sizeof(double));
  L->b = (double*)calloc((size_t)n, sizeof(double));
  L->r = (double*)calloc((size_t)n, sizeof(double));
  L->d = (double*)calloc((size_t)n, sizeof(double));
  L->t = (double*)calloc((size_t)n, sizeof(double));
}

static void apply(const Level* L, const double* x, double* y) {
  const int nx = L->nx, ny = L->ny, P = nx + 1;
  for (int i = 0; i <= ny; ++i)
    for (int j = 0; j <= nx; ++j) {
      const int k = j + i * P;
      const double* s = L->st + 7 * (size_t)k;
      double v = s[0] * x[k];
      if (j < nx) v += s[1] * x[k + 1];
      if (j > 0) v += s[2] * x[k - 1];
      if (i < ny) v += s[3] * x[k + P];
      if (i > 0) v += s[4] * x[k - P];
      if (i < ny && j < nx) v += s[5] * x[k + P + 1];
      if (i > 0 && j > 0) v += s[6] * x[k - P - 1];
      y[k] = v;
    }
}

static void coarsest_factor(Level* L) {
  const int P = L->nx + 1, n = P * (L->ny + 1);
  L->freeidx = (int*)malloc(sizeof(int) * (size_t)n);
  int m = 0;
  for (int k = 0; k < n; ++k)
    if (!L->dir[k]) L->freeidx[m++] = k;
  L->nfree = m;
  double* A = (double*)calloc((size_t)m * m, sizeof(double));
  int* pos = (int*)malloc(sizeof(int) * (size_t)n);
  for (int k = 0; k < n; ++k) pos[k] = -1;
  for (int q = 0; q < m; ++q) pos[L->freeidx[q]] = q;
  double* e = (double*)calloc((size_t)n, sizeof(double));
  double* col = (double*)calloc((size_t)n, sizeof(double));
  for (int q = 0; q < m; ++q) {
    e[L->freeidx[q]] = 1.0;
    apply(L, e, col);
    e[L->freeidx[q]] = 0.0;
    for (int k = 0; k < n; ++k)
      if (pos[k] >= 0) A[(size_t)pos[k] * m + q] = col[k];
  }
  for (int c = 0; c < m; ++c) { /* Cholesky, lower triangle in place */
    double s = A[(size_t)c * m + c];
    for (int k = 0; k < c; ++k) s -= A[(size_t)c * m + k] * A[(size_t)c * m + k];
    const double dcc = sqrt(s);
    A[(size_t)c * m + c] = dcc;
    for (int r = c + 1; r < m; ++r) {
      double v = A[(size_t)r * m + c];
      for (int k = 0; k < c; ++k) v -= A[(size_t)r * m + k] * A[(size_t)c * m + k];
      A[(size_t)r * m + c] = v / dcc;
    }
  }
  L->chol = A;
  free(pos);
  free(e);
  free(col);
}

static void coarsest_solve(const Level* L, const double* b, double* x) {
  const int m = L->nfree, n = (L->nx + 1) * (L->ny + 1);
  double* y = L->t;
  for (int q = 0; q < m; ++q) {
    double v = b[L->freeidx[q]];
    for (int k = 0; k < q; ++k) v -= L->chol[(size_t)q * m + k] * y[k];
    y[q] = v / L->chol[(size_t)q * m + q];
  }
  for (int q = m - 1; q >= 0; --q) {
    double v = y[q];
    for (int k = q + 1; k < m; ++k) v -= L->chol[(size_t)k * m + q] * y[k];
    y[q] = v / L->chol[(size_t)q * m + q];
  }
  for (int k = 0; k < n; ++k) x[k] = 0.0;
  for (int q = 0; q < m; ++q) x[L->freeidx[q]] = y[q];
}

/* 1-D interpolation from a coarse axis: fine node f between coarse nodes lo, lo+1
 * with weight w on lo+1 */
static void axis_map(const double* fx, int nf, const double* cx, int nc, int f, int* lo, double* w) {
  if (nc == nf) {
    *lo = f;
    *w = 0.0;
    return;
  }
  if (f == nf) {
    *lo = nc;
    *w = 0.0;
    return;
  }
  if ((f & 1) == 0) {
    *lo = f / 2;
    *w = 0.0;
    return;
  }
  const int J = (f - 1) / 2;
  *lo = J;
  *w = (fx[f] - cx[J]) / (cx[J + 1] - cx[J]);
}

/* y_f += P x_c (ADD) or y_c = P^T x_f (transpose) */
static void prolong(const Level* F, const Level* Cc, const double* xc, double* yf) {
  const int Pf = F->nx + 1, Pc = Cc->nx + 1;
  for (int i = 0; i <= F->ny; ++i) {
    int il;
    double wi;
    axis_map(F->ys, F->ny, Cc->ys, Cc->ny, i, &il, &wi);
    for (int j = 0; j <= F->nx; ++j) {
      int jl;
      double wj;
      axis_map(F->xs, F->nx, Cc->xs, Cc->nx, j, &jl, &wj);
      const int k = j + i * Pf;
      if (F->dir[k]) continue;
      double v = (1 - wi) * (1 - wj) * xc[jl + il * Pc];
      if (wj > 0) v += (1 - wi) * wj * xc[jl + 1 + il * Pc];
      if (wi > 0) v += wi * (1 - wj) * xc[jl + (il + 1) * Pc];
      if (wi > 0 && wj > 0) v += wi * wj * xc[jl + 1 + (il + 1) * Pc];
      yf[k] += v;
    }
  }
}

static void restrict_t(const Level* F, const Level* Cc, const double* rf, double* bc) {
  const int Pf = F->nx + 1, Pc = Cc->nx + 1, nc = Pc * (Cc->ny + 1);
  for (int k = 0; k < nc; ++k) bc[k] = 0.0;
  for (int i = 0; i <= F->ny; ++i) {
    int il;
    double wi;
    axis_map(F->ys, F->ny, Cc->ys, Cc->ny, i, &il, &wi);
    for (int j = 0; j <= F->nx; ++j) {
      int jl;
      double wj;
      axis_map(F->xs, F->nx, Cc->xs, Cc->nx, j, &jl, &wj);
      const int k = j + i * Pf;
      if (F->dir[k]) continue;
      const double r = rf[k];
      bc[jl + il * Pc] += (1 - wi) * (1 - wj) * r;
      if (wj > 0) bc[jl + 1 + il * Pc] += (1 - wi) * wj * r;
      if (wi > 0) bc[jl + (il + 1) * Pc] += wi * (1 - wj) * r;
      if (wi > 0 && wj > 0) bc[jl + 1 + (il + 1) * Pc] += wi * wj * r;
    }
  }
  for (int k = 0; k < nc; ++k)
    if (Cc->dir[k]) bc[k] = 0.0;
}

/* deg Chebyshev-Jacobi steps on [lmax/5, lmax] from x (zero when from_zero) */
static void chebyshev(const Level* L, const double* b, double* x, int deg, int from_zero) {
  const int n = (L->nx + 1) * (L->ny + 1);
  const double lmax = L->lmax, lmin = lmax / 5.0;
  const double theta = 0.5 * (lmax + lmin), delta = 0.5 * (lmax - lmin), sigma = theta / delta;
  double rho_old = 1.0 / sigma;
  double* r = L->r;
  double* d = L->d;
  if (from_zero)
    for (int k = 0; k < n; ++k) r[k] = b[k];
  else {
    apply(L, x, r);
    for (int k = 0; k < n; ++k) r[k] = b[k] - r[k];
  }
  for (int k = 0; k < n; ++k) {
    d[k] = L->idg[k] * r[k] / theta;
    x[k] = (from_zero ? 0.0 : x[k]) + d[k];
  }
  for (int s = 1; s < deg; ++s) {
    apply(L, x, r);
    const double rho = 1.0 / (2.0 * sigma - rho_old);
    for (int k = 0; k < n; ++k) {
      d[k] = rho * rho_old * d[k] + 2.0 * rho / delta * L->idg[k] * (b[k] - r[k]);
      x[k] += d[k];
    }
    rho_old = rho;
  }
}

static void vcycle(Hier* Hh, int l, const double* b, double* x) {
  Level* L = &Hh->L[l];
  const int n = (L->nx + 1) * (L->ny + 1);
  if (l == Hh->nlev - 1) {
    coarsest_solve(L, b, x);
    return;
  }
  Level* C = &Hh->L[l + 1];
  chebyshev(L, b, x, 2, 1);
  apply(L, x, L->r);
  for (int k = 0; k < n; ++k) L->r[k] = L->dir[k] ? 0.0 : b[k] - L->r[k];
  restrict_t(L, C, L->r, C->b);
  vcycle(Hh, l + 1, C->b, C->x);
  prolong(L, C, C->x, x);
  chebyshev(L, b, x, 2, 0);
}

static void hier_free(Hier* H) {
  for (int l = 0; l < H->nlev; ++l) {
    Level* L = &H->L[l];
    free(L->xs); free(L->ys); free(L->st); free(L->idg); free(L->dir);
    free(L->x); free(L->b); free(L->r); free(L->d); free(L->t);
    free(L->chol); free(L->freeidx);
  }
}

static void hier_build(Hier* H, int nx, int ny, double W, double Hh, double D, double dt,
                       double g, unsigned walls) {
  memset(H, 0, sizeof(*H));
  H->alpha = 1.0 + dt * g;
  H->beta = dt * D;
  int l = 0;
  Level* L = &H->L[0];
  L->nx = nx;
  L->ny = ny;
  L->xs = (double*)malloc(sizeof(double) * (size_t)(nx + 1));
  L->ys = (double*)malloc(sizeof(double) * (size_t)(ny + 1));
  for (int j = 0; j <= nx; ++j) L->xs[j] = W * (double)j / nx;
  for (int i = 0; i <= ny; ++i) L->ys[i] = Hh * (double)i / ny;
  for (;;) {
    build_level(&H->L[l], H->alpha, H->beta, walls);
    const int cx = coarse_count(H->L[l].nx), cy = coarse_count(H->L[l].ny);
    const int small = (H->L[l].nx + 1) * (H->L[l].ny + 1) <= 300;
    if ((cx == H->L[l].nx && cy == H->L[l].ny) || l + 1 == MAXLEV || small) break;
    Level* C = &H->L[l + 1];
    C->nx = cx;
    C->ny = cy;
    C->xs = (double*)malloc(sizeof(double) * (size_t)(cx + 1));
    C->ys = (double*)malloc(sizeof(double) * (size_t)(cy + 1));
    coarse_positions(H->L[l].xs, H->L[l].nx, C->xs, cx);
    coarse_positions(H->L[l].ys, H->L[l].ny, C->ys, cy);
    ++l;
  }
  H->nlev = l + 1;
  coarsest_factor(&H->L[l]);
}

static double dot(const double* a, const double* b, int n) {
  double s = 0.0;
  for (int k = 0; k < n; ++k) s += a[k] * b[k];
  return s;
}

/* mass rows on the finest (uniform) level */
static void mass_apply(const Level* L, const double* u, double* y) {
  const int nx = L->nx, ny = L->ny, P = nx + 1;
  const double hx = L->xs[1] - L->xs[0], hy = L->ys[1] - L->ys[0];
  for (int i = 0; i <= ny; ++i)
    for (int j = 0; j <= nx; ++j) {
      const int k = j + i * P;
      const double hxl = j > 0 ? hx : 0, hxr = j < nx ? hx : 0, hyd = i > 0 ? hy : 0,
                   hyu = i < ny ? hy : 0, sx = hxl + hxr, sy = hyd + hyu;
      double v = (2 * hxl * hyd + hxr * hyd + hxl * hyu + 2 * hxr * hyu) / 12.0 * u[k];
      if (j < nx) v += hxr * sy / 24.0 * u[k + 1];
      if (j > 0) v += hxl * sy / 24.0 * u[k - 1];
      if (i < ny) v += hyu * sx / 24.0 * u[k + P];
      if (i > 0) v += hyd * sx / 24.0 * u[k - P];
      if (i < ny && j < nx) v += hxr * hyu / 12.0 * u[k + P + 1];
      if (i > 0 && j > 0) v += hxl * hyd / 12.0 * u[k - P - 1];
      y[k] = v;
    }
}

/* steps of one trap; u (grid order) in/out; returns CG iterations */
static long long trap_steps(int nx, int ny, double W, double H, double D, double dt, double g,
                            unsigned walls, const double* F, double* u, int steps, double rtol,
                            double budget_s, int* done, double* step_seconds) {
  Hier Hh;
  hier_build(&Hh, nx, ny, W, H, D, dt, g, walls);
  Level* L = &Hh.L[0];
  const int n = (nx + 1) * (ny + 1);
  double* b = (double*)malloc(sizeof(double) * (size_t)n);
  double* r = (double*)malloc(sizeof(double) * (size_t)n);
  double* z = (double*)malloc(sizeof(double) * (size_t)n);
  double* p = (double*)malloc(sizeof(double) * (size_t)n);
  double* q = (double*)malloc(sizeof(double) * (size_t)n);
  long long iters = 0;
  const double t0 = now_s();
  *done = 0;
  for (int s = 0; s < steps; ++s) {
    mass_apply(L, u, b);
    for (int k = 0; k < n; ++k) b[k] = L->dir[k] ? 0.0 : b[k] + F[k];
    for (int k = 0; k < n; ++k)
      if (L->dir[k]) u[k] = 0.0;
    const double bb = dot(b, b, n);
    apply(L, u, r);
    for (int k = 0; k < n; ++k) r[k] = b[k] - r[k];
    double rr = dot(r, r, n);
    if (rr > rtol * rtol * bb && bb > 0) {
      memset(z, 0, sizeof(double) * (size_t)n);
      vcycle(&Hh, 0, r, z);
      memcpy(p, z, sizeof(double) * (size_t)n);
      double rz = dot(r, z, n);
      for (int it = 0; it < 200; ++it) {
        apply(L, p, q);
        const double alpha = rz / dot(p, q, n);
        for (int k = 0; k < n; ++k) {
          u[k] += alpha * p[k];
          r[k] -= alpha * q[k];
        }
        ++iters;
        rr = dot(r, r, n);
        if (rr <= rtol * rtol * bb) break;
        memset(z, 0, sizeof(double) * (size_t)n);
        vcycle(&Hh, 0, r, z);
        const double rz2 = dot(r, z, n);
        const double beta = rz2 / rz;
        rz = rz2;
        for (int k = 0; k < n; ++k) p[k] = z[k] + beta * p[k];
      }
    }
    *done += 1;
    if (now_s() - t0 > budget_s) break;
  }
  *step_seconds = now_s() - t0;
  free(b); free(r); free(z); free(p); free(q);
  hier_free(&Hh);
  return iters;
}

/* Every trap of a sample in parallel (one per thread): trap t has params par[8t..8t+7]
 * = (nx, ny, W, H, D, dt, g, walls), its load and field at offset off[t] of F and u.
 * Returns the DOF-steps done; *seconds the wall time of the parallel region, *threads
 * the threads used and trap_seconds[t] the time of trap t's steps (its multigrid
 * hierarchy and coarsest factor, built once, excluded). */
long long gmg_cpu_batch(int ntraps, const double* par, const long long* off, const double* F,
                        double* u, int steps, double rtol, double budget_s, int nthreads,
                        double* seconds, int* threads, long long* iters_out,
                        double* trap_seconds) {
  long long dofs = 0, iters = 0;
  int used = 1;
  const double t0 = now_s();
#ifdef _OPENMP
  if (nthreads > 0) omp_set_num_threads(nthreads);
#endif
#pragma omp parallel reduction(+ : dofs, iters)
  {
#ifdef _OPENMP
#pragma omp single
    used = omp_get_num_threads();
#endif
#pragma omp for schedule(dynamic, 1)
    for (int t = 0; t < ntraps; ++t) {
      const double* q = par + 8 * (size_t)t;
      const int nx = (int)q[0], ny = (int)q[1];
      int done = 0;
      iters += trap_steps(nx, ny, q[2], q[3], q[4], q[5], q[6], (unsigned)q[7], F + off[t],
                          u + off[t], steps, rtol, budget_s, &done, &trap_seconds[t]);
      dofs += (long long)(nx + 1) * (ny + 1) * done;
    }
  }
  *seconds = now_s() - t0;
  *threads = used;
  *iters_out = iters;
  return dofs;
}
