// FP64 total-HSL mass balance of every step, on the device.
//
// The step solves, on the free rows, A c' = M c + F with the full operator
// A = alpha M + dt D K + dt C + R (alpha = 1 + dt g; K the stiffness, C the Galerkin
// advection, R the Robin facet terms), the load F of the point cells and Robin walls,
// and the Dirichlet rows held at their wall values.  Summing the full system over
// every row gives the discrete balance of the step:
//
//   alpha 1'M c' + 1'(dt C + R) c' - 1'M c - 1'F = sum over Dirichlet rows of
//   (A c' - M c - F) + sum over free rows of (A c' - M c - F)
//
// because the stiffness rows and columns sum to zero for any tensor.  The first sum
// on the right is the consistent (residual) flux through the Dirichlet walls; the
// second is the solver's residual, zero up to the step's tolerance.  So
//
//   mass' - mass = load - decay - operator loss - wall outflow + drift
//
// with decay = dt g 1'M c', the operator loss 1'(dt C + R) c' (advective outflow and
// the Robin walls' outflow), the wall outflow minus the Dirichlet rows' sum and the
// drift the free rows' residual sum.  1'M c is the lumped-mass sum (the mass rows sum
// to the nodes' shares of the triangle areas), so the balance reads each field once.
// The reference keeps only the facet functional -int grad c . n ds of the new field
// (fenics/boundary.ufl:9-12, src/fHSL.cpp:156-160); that is the same outflow up to
// the discretisation error, not to rounding, so the drift is formed with the
// consistent flux.
#pragma once
#include "eqf_common.cuh"
#include "eqf_kernels.cuh"
#include "eqf_walls.cuh"

namespace eqf {

constexpr int kBalFields = 12;
// per trap record (FP64), the eqf_balance fields in order
enum : int {
  BAL_MASS = 0, BAL_MASS_PREV, BAL_LOAD, BAL_DECAY, BAL_OPERATOR, BAL_WALL, BAL_DRIFT,
  BAL_DRIFT_SUM, BAL_DRIFT_ABS_SUM, BAL_LOAD_SUM, BAL_DRIFT_REL_MAX, BAL_STEPS
};

// Index of node (i, j) in the rim arrays of k_wall_rim (rim_node's inverse), -1 off
// the rim.
__device__ __forceinline__ int rim_index(int i, int j, int nx, int ny) {
  if (i < 2) return i * (nx + 1) + j;
  if (i > ny - 2) return (i - ny + 3) * (nx + 1) + j;
  if (j < 2) return 4 * (nx + 1) + (i - 2) * 4 + j;
  if (j > nx - 2) return 4 * (nx + 1) + (i - 2) * 4 + (j - nx + 3);
  return -1;
}

// Lumped mass of node (i, j) on the finest (uniform) level: the node's share of its
// triangles' areas, 1/3 of each; hx*hy for every node off the boundary.
__device__ __forceinline__ double lumped_mass(const LevelGeom& g, int i, int j) {
  const double hxl = j > 0 ? g.hx : 0.0, hxr = j < g.nx ? g.hx : 0.0;
  const double hyd = i > 0 ? g.hy : 0.0, hyu = i < g.ny ? g.hy : 0.0;
  return (2.0 * hxl * hyd + hxr * hyd + hxl * hyu + 2.0 * hxr * hyu) * (1.0 / 6.0);
}

// Column sum of the advection operator dt*C at node (i, j): dt * int v . grad phi_j,
// with dt*v = (0, -adv*y) P1, taken over the squares around the node (each square's
// lower-right and upper-left triangles weigh dt*v_y by their vertices' mean).  Off
// the boundary it is adv*hx*hy (minus the divergence of dt*v times the node's area).
__device__ __forceinline__ double adv_column(const LevelGeom& g, int i, int j) {
  auto v1 = [&](int r) { return -g.adv * g.hy * (3.0 * r + 1.0) * (1.0 / 3.0); };  // (2y_r + y_r+1)/3
  auto v2 = [&](int r) { return -g.adv * g.hy * (3.0 * r + 2.0) * (1.0 / 3.0); };  // (y_r + 2y_r+1)/3
  double w = 0.0;
  if (i < g.ny && j < g.nx) w -= v2(i);
  if (i < g.ny && j > 0) w -= v1(i);
  if (i > 0 && j < g.nx) w += v2(i - 1);
  if (i > 0 && j > 0) w += v1(i - 1);
  return 0.5 * g.hx * w;
}

// Robin walls' column sum at a boundary node: dt*r*|e|/2 per facet end.
__device__ __forceinline__ double robin_column(const LevelGeom& g, int i, int j) {
  const double hxs = ((j > 0 ? g.hx : 0.0) + (j < g.nx ? g.hx : 0.0)) * 0.5;
  const double hys = ((i > 0 ? g.hy : 0.0) + (i < g.ny ? g.hy : 0.0)) * 0.5;
  double rc = 0.0;
  if (i == 0) rc += g.rob[0] * hxs;
  if (i == g.ny) rc += g.rob[1] * hxs;
  if (j == 0) rc += g.rob[2] * hys;
  if (j == g.nx) rc += g.rob[3] * hys;
  return rc;
}

// The load of rim node (i, j) before any Dirichlet lifting, for a trap whose walls
// carry values or Robin loads (its F was rewritten on the rim; the point cells' part
// is kept in fbase).
__device__ __forceinline__ double rim_load(const LevelGeom& g, const WallDev& w,
                                           const double* __restrict__ fbase, int r, int i,
                                           int j) {
  double f = fbase[w.rim0 + r];
  const double hxl = j > 0 ? g.hx : 0.0, hxr = j < g.nx ? g.hx : 0.0;
  const double hyd = i > 0 ? g.hy : 0.0, hyu = i < g.ny ? g.hy : 0.0;
  if (i == 0) f += w.robs[EQF_SIDE_BOTTOM] * (hxl + hxr) * 0.5;
  if (i == g.ny) f += w.robs[EQF_SIDE_TOP] * (hxl + hxr) * 0.5;
  if (j == 0) f += w.robs[EQF_SIDE_LEFT] * (hyd + hyu) * 0.5;
  if (j == g.nx) f += w.robs[EQF_SIDE_RIGHT] * (hyd + hyu) * 0.5;
  return f;
}

constexpr int kBalTileParts = 3;  // per row tile: sum c', sum c, sum F (raw, every node)
constexpr int kBalRimParts = 5;   // per rim block: the boundary corrections

// Streaming pass (finest-level row tiles): the plain sums of c', c and F over the
// tile's nodes, 4-node vectors per thread, the pad columns masked.  Every node off
// the boundary weighs hx*hy in the mass and adv*hx*hy in the advection term, so the
// weights are applied once per trap; the boundary's own weights are corrections
// added by k_balance_rim.  OLD = false / LOAD = false leave out c / F when the
// previous step's mass / load still hold (the finish kernel carries them over).
template <bool OLD, bool LOAD>
__global__ void __launch_bounds__(kThreads)
    k_balance_tiles(const LevelGeom* __restrict__ G, const Tile* __restrict__ tiles,
                    const double* __restrict__ un, const double* __restrict__ uo,
                    const double* __restrict__ F, const int* __restrict__ frozen,
                    double* __restrict__ part) {
  const Tile tile = tiles[blockIdx.x];
  const LevelGeom& g = G[tile.geom];
  double* out = part + (size_t)blockIdx.x * kBalTileParts;
  const int trap = g.trap, P = g.P, nx = g.nx;
  if (frozen[trap]) {
    if (threadIdx.x < kBalTileParts) out[threadIdx.x] = 0.0;
    return;
  }
  const long long base = g.off + (long long)tile.r0 * P;
  const double* a = un + base;
  const double* b = uo + base;
  const double* f = F + base;
  const int qpr = P >> 2, nq = (tile.r1 - tile.r0) * qpr;
  // 4-node vectors over the tile's rows, two quads per thread and pass in two
  // independent accumulators
  double sa0 = 0.0, sa1 = 0.0, sb0 = 0.0, sb1 = 0.0, sf0 = 0.0, sf1 = 0.0;
  auto quad = [&](int q, double& xa, double& xb, double& xf) {
    const int row = q / qpr, j0 = (q - row * qpr) * 4, k = row * P + j0;
    Q4<double> x = vld4<double>(a + k), y{}, z{};
    if (OLD) y = vld4<double>(b + k);
    if (LOAD) z = vld4<double>(f + k);
    if (j0 + 3 > nx) {
#pragma unroll
      for (int e = 0; e < 4; ++e)
        if (j0 + e > nx) x.v[e] = y.v[e] = z.v[e] = 0.0;
    }
    xa += (x.v[0] + x.v[1]) + (x.v[2] + x.v[3]);
    if (OLD) xb += (y.v[0] + y.v[1]) + (y.v[2] + y.v[3]);
    if (LOAD) xf += (z.v[0] + z.v[1]) + (z.v[2] + z.v[3]);
  };
  for (int q = threadIdx.x; q < nq; q += 2 * kThreads) {
    quad(q, sa0, sb0, sf0);
    if (q + kThreads < nq) quad(q + kThreads, sa1, sb1, sf1);
  }
  const double v[kBalTileParts] = {sa0 + sa1, sb0 + sb1, sf0 + sf1};
#pragma unroll
  for (int p = 0; p < kBalTileParts; ++p) {
    const double t = block_sum(v[p]);
    if (threadIdx.x == 0) out[p] = t;
  }
}

// Boundary pass, blockIdx.y = trap: over the outer ring of nodes, the corrections of
// the lumped mass and of the advection column sum to their off-boundary values, the
// Robin column sums and, on Dirichlet rows, the full operator's residual; over the
// two-node rim of a trap whose walls carry values or Robin loads, the load before
// lifting minus the F the tile pass summed.
__global__ void __launch_bounds__(kThreads, 2)
    k_balance_rim(const LevelGeom* __restrict__ G, const double* __restrict__ un,
                  const double* __restrict__ uo, const double* __restrict__ F,
                  const int* __restrict__ wall_of, const WallDev* __restrict__ walls,
                  const double* __restrict__ fbase, const int* __restrict__ frozen,
                  int old, int load, double* __restrict__ part) {
  const int t = blockIdx.y;
  const LevelGeom& g = G[t];
  double* out = part + ((size_t)t * gridDim.x + blockIdx.x) * kBalRimParts;
  double dm = 0.0, dmo = 0.0, dop = 0.0, df = 0.0, dw = 0.0;
  if (!frozen[t]) {
    const int nx = g.nx, ny = g.ny, P = g.P;
    const double* a = un + g.off;
    const double* b = uo + g.off;
    const double* Fs = F + g.off;
    const double hxy = g.hx * g.hy, adv_in = g.adv * hxy;
    const int wi = wall_of[t];
    const int ring = 2 * (nx + 1) + 2 * (ny - 1);
    const int rim = wi >= 0 && load ? rim_count(nx, ny) : 0;
    const int n = ring > rim ? ring : rim;
    for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < n; r += gridDim.x * blockDim.x) {
      if (r < ring) {
        int i, j;
        if (r < nx + 1) {
          i = 0;
          j = r;
        } else if (r < 2 * (nx + 1)) {
          i = ny;
          j = r - (nx + 1);
        } else {
          const int q = r - 2 * (nx + 1);
          i = 1 + (q >> 1);
          j = (q & 1) ? nx : 0;
        }
        const int k = i * P + j;
        const double an = a[k], ao = b[k];
        const double dmass = lumped_mass(g, i, j) - hxy;
        dm = fma(dmass, an, dm);
        if (old) dmo = fma(dmass, ao, dmo);
        double opw = robin_column(g, i, j);
        if (g.adv_on) opw += adv_column(g, i, j) - adv_in;
        if (opw != 0.0) dop = fma(opw, an, dop);
        if (g.walls && is_dirichlet(g, i, j)) {
          // the full operator's row (no Dirichlet reduction) on c', the mass row on c,
          // the load before lifting
          const double fk = wi >= 0 ? rim_load(g, walls[wi], fbase, rim_index(i, j, nx, ny), i, j)
                                    : Fs[k];
          const Sten<double> s = stencil_general<double, true, false>(g, i, j);
          const Sten<double> m = mass_stencil<double>(g, i, j);
          double res = s.c * an - m.c * ao - fk;
          if (j < nx) res += s.e * a[k + 1] - m.e * b[k + 1];
          if (j > 0) res += s.w * a[k - 1] - m.w * b[k - 1];
          if (i < ny) res += s.n * a[k + P] - m.n * b[k + P];
          if (i > 0) res += s.s * a[k - P] - m.s * b[k - P];
          if (i < ny && j < nx) res += s.ne * a[k + P + 1] - m.ne * b[k + P + 1];
          if (i > 0 && j > 0) res += s.sw * a[k - P - 1] - m.sw * b[k - P - 1];
          dw += res;
        }
      }
      if (r < rim) {  // the load before lifting on the two-node rim
        int i, j;
        rim_node(r, nx, ny, i, j);
        const int k = i * P + j;
        df += rim_load(g, walls[wi], fbase, r, i, j) - Fs[k];
      }
    }
  }
  const double v[kBalRimParts] = {dm, dmo, dop, df, dw};
#pragma unroll
  for (int p = 0; p < kBalRimParts; ++p) {
    const double s = block_sum(v[p]);
    if (threadIdx.x == 0) out[p] = s;
  }
}

// One warp per trap: lane l sums the partials l, l + 32, ... in order, then a fixed
// shuffle tree (the figures depend on the trap's own tile count only, not on the
// batch), then lane 0 writes the trap's record.  old / load = 0 take the previous
// step's mass as this step's starting mass / its load as this step's.
__device__ __forceinline__ double warp_total(double v) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}
__global__ void k_balance_finish(const LevelGeom* __restrict__ G,
                                 const TileRange* __restrict__ range,
                                 const double* __restrict__ tpart, const double* __restrict__ rpart,
                                 int rim_blocks, const int* __restrict__ frozen, int ntraps,
                                 int old, int load, double* __restrict__ rec) {
  const int t = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5), lane = threadIdx.x & 31;
  if (t >= ntraps || frozen[t]) return;
  const TileRange tr = range[t];
  double s[kBalTileParts] = {0.0, 0.0, 0.0};
  for (int q = lane; q < tr.count; q += 32)
    for (int p = 0; p < kBalTileParts; ++p) s[p] += tpart[(size_t)(tr.first + q) * kBalTileParts + p];
  double c[kBalRimParts] = {0.0, 0.0, 0.0, 0.0, 0.0};
  for (int q = lane; q < rim_blocks; q += 32)
    for (int p = 0; p < kBalRimParts; ++p)
      c[p] += rpart[((size_t)t * rim_blocks + q) * kBalRimParts + p];
  for (int p = 0; p < kBalTileParts; ++p) s[p] = warp_total(s[p]);
  for (int p = 0; p < kBalRimParts; ++p) c[p] = warp_total(c[p]);
  if (lane != 0) return;
  const LevelGeom& g = G[t];
  double* r = rec + (size_t)t * kBalFields;
  const double hxy = g.hx * g.hy;
  const double mass = fma(hxy, s[0], c[0]);
  const double prev = old ? fma(hxy, s[1], c[1]) : r[BAL_MASS];
  const double ld = load ? s[2] + c[3] : r[BAL_LOAD];
  const double op = fma(g.adv * hxy, s[0], c[2]);
  const double decay = (g.alpha - 1.0) * mass;
  const double wall = -c[4];
  const double drift = mass - prev - ld + decay + op + wall;
  r[BAL_MASS] = mass;
  r[BAL_MASS_PREV] = prev;
  r[BAL_LOAD] = ld;
  r[BAL_DECAY] = decay;
  r[BAL_OPERATOR] = op;
  r[BAL_WALL] = wall;
  r[BAL_DRIFT] = drift;
  r[BAL_DRIFT_SUM] += drift;
  r[BAL_DRIFT_ABS_SUM] += fabs(drift);
  r[BAL_LOAD_SUM] += ld;
  // relative to the largest of the step's terms
  const double scale = fmax(fmax(fabs(mass), fabs(prev)), fmax(fabs(ld), fabs(wall)));
  if (scale > 0.0) r[BAL_DRIFT_REL_MAX] = fmax(r[BAL_DRIFT_REL_MAX], fabs(drift) / scale);
  r[BAL_STEPS] += 1.0;
}

}  // namespace eqf
