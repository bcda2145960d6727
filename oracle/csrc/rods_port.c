/*
 * Plain-C restatement of eQ's rod-cell coupling loop (the timed CPU baseline of the
 * rod exchange, and a second restatement checked against the reference's own code).
 *
 * TEST/BENCH INFRASTRUCTURE ONLY: tests and the CPU legs of bench.py call it; the
 * product never does.  It follows oracle/rods.py operation by operation (built with
 * -ffp-contract=off, so every double operation rounds on its own, as in the
 * reference): findInteriorPoints (src/abm/eQabm.cpp:268-304) with
 * cpmEcoli::pointIsInCell (src/abm/cpmEcoli.cpp:313-328) and chipmunk 7.0.1's
 * cpBodyWorldToLocal, readHSL (eQabm.cpp:326-337), the strain's membrane exchange
 * (src/Strain.h:281-345, src/Strain.cpp:10-83) and writeHSL (eQabm.cpp:338-359) with
 * the eQ::Cell conversions (src/eQcell.h:42-97).  Cells run one after the other.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>

#define ROD_DOUBLES 20 /* the eqf_rod record */
enum { HELD = 0, CIRCUIT = 1, INERT = 2 };

static const double kWidth = 1.0;

static int c_round(double x) { /* x >= 0, half away from zero */
  const double f = floor(x);
  return (int)f + (x - f >= 0.5 ? 1 : 0);
}

static int inside(const double* r, double x, double y) {
  const double c = r[8], s = r[9], px = r[6], py = r[7];
  const double tx = (-s) * py - px * c, ty = px * s - c * py;
  const double lx = (c * x + s * y) + tx, ly = ((-s) * x + c * y) + ty;
  const double* v = r + 10;
  for (int k = 0; k < 4; ++k) {
    const int n = (k + 1) & 3;
    const double ex = v[2 * n] - v[2 * k], ey = v[2 * n + 1] - v[2 * k + 1];
    const double qx = lx - v[2 * n], qy = ly - v[2 * n + 1];
    if (!(ex * qy - ey * qx < 0.0)) return 0;
  }
  return 1;
}

/* footprint of one cell into nodes[] (grid index i*(nx+1)+j), returns the count */
static int footprint(const double* r, double npm, int nx, int ny, int* nodes, int cap) {
  const int nte = c_round(npm * kWidth / 2.0);
  const int ai = c_round(r[3] * npm), aj = c_round(r[2] * npm);
  const int bi = c_round(r[5] * npm), bj = c_round(r[4] * npm);
  int i1 = ai > bi ? bi : ai, i2 = ai > bi ? ai : bi;
  int j1 = aj > bj ? bj : aj, j2 = aj > bj ? aj : bj;
  i1 = i1 >= nte ? i1 - nte : 0;
  j1 = j1 >= nte ? j1 - nte : 0;
  i2 = i2 + nte >= ny ? ny : i2 + nte;
  j2 = j2 + nte >= nx ? nx : j2 + nte;
  int k = 0;
  for (int i = i1; i <= i2; ++i)
    for (int j = j1; j <= j2; ++j)
      if (inside(r, (double)j / npm, (double)i / npm)) {
        if (k < cap) nodes[k] = i * (nx + 1) + j;
        ++k;
      }
  if (k == 0) {
    nodes[0] = c_round(r[1] * npm) * (nx + 1) + c_round(r[0] * npm);
    k = 1;
  }
  return k;
}

/* One pass over the cells.  fields: nl grids of (ny+1)*(nx+1), updated in place;
 * ihsl / ehsl / prod / mode: n*nl cell-major.  Returns 0, or -1 when a footprint
 * exceeds the scratch. */
int rods_port_exchange(int nx, int ny, double npm, double dt, const double* km, int nl, int n,
                       const double* rods, double* ihsl, const double* prod,
                       const uint8_t* mode, double* fields, double* ehsl, int* points) {
  const double pi = 3.14159265358979323846;
  const double r0 = kWidth / 2.0;
  const double cyl = pi * (r0 * r0), pole = 4.0 / 3.0 * pi * (r0 * r0 * r0);
  const double k_nm = 1.0 / 0.602;
  const size_t nn = (size_t)(nx + 1) * (ny + 1);
  const int cap = (nx + 1) * (ny + 1);
  int* nodes = (int*)malloc(sizeof(int) * (size_t)cap);
  if (!nodes) return -1;
  for (int c = 0; c < n; ++c) {
    const double* r = rods + (size_t)ROD_DOUBLES * c;
    const int K = footprint(r, npm, nx, ny, nodes, cap);
    if (K > cap) {
      free(nodes);
      return -1;
    }
    points[c] = K;
    const double L = r[18];
    const double V = (L - kWidth) * cyl + pole;
    const double nmpm = (1.0 / V) * k_nm;
    const double ecf = 1.0 - V / (L * 1.0 * 1.0);
    for (int l = 0; l < nl; ++l) {
      double* u = fields + (size_t)l * nn;
      double acc = 0.0;
      for (int k = 0; k < K; ++k) acc += u[nodes[k]];
      const double e = acc / (double)K;
      const size_t s = (size_t)c * nl + l;
      ehsl[s] = e;
      if (mode[s] == INERT) continue;
      const double inm = ihsl[s] * nmpm;
      const double dH = dt * (km[l] * (inm - e));
      const double delta = mode[s] == CIRCUIT ? dt * prod[s] - dH : 0.0;
      double inew = inm + delta;
      if (inew < 0.0) inew = 0.0;
      ihsl[s] = inew / nmpm;
      const double number = dH / k_nm * V;
      const double per_um2 = number / ecf;
      const double d = per_um2 * npm * npm / (double)K;
      for (int k = 0; k < K; ++k) u[nodes[k]] += d;
    }
  }
  free(nodes);
  return 0;
}
