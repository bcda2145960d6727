// Wall conditions with values and the flow channels of the MICROFLUIDIC_TRAP mode.
//
// Non-zero Dirichlet values and Robin loads enter the step through the load vector
// F on the trap's rim (the nodes within one node of a wall): a Dirichlet row takes
// b = its value (its operator row is the identity), and every other rim row
// subtracts the couplings of the full operator to its Dirichlet neighbours times
// their values (the lifting that makes the reduced, symmetric operator -- couplings
// to Dirichlet nodes removed -- give DOLFIN's row-replaced solution,
// src/fHSL.cpp:104-106 with the DirichletBCs of 446-540) and adds the Robin load
// dt*r*s*|e|/2 per facet end (fenics/hslD.ufl:36-42).  F's rim values from the point
// cells are kept apart (fbase) so the rim can be rewritten every step as the
// channels change.
//
// A flow channel (fenicsChannel, src/fHSL.h:240-330) is the P1 Crank-Nicolson
// advection-diffusion form of fenics/AdvectionDiffusion.ufl on the nx+1 nodes of
// the wall: (M + dt_c/2 (D K + v C) + dt_c/2 R) c' = (M - dt_c/2 (D K + v C) -
// dt_c/2 R) c, R the Robin rates at its two ends (s = 0).  After the trap solve each
// channel takes the flux h*(dt*D*grad_j)/well_scaling of every column
// (computeBoundaryFlux, src/fHSL.cpp:54-95) in `substeps` equal parts, one before
// each sub-step (stepDiffusion, src/fHSL.cpp:110-140).  The sub-step's tridiagonal
// solve is parallel cyclic reduction with its multipliers precomputed on the host
// (the matrix is the same every sub-step): per level d_i -= k1_i d_{i-s} + k2_i d_{i+s}.
#pragma once
#include "eqf_common.cuh"
#include "../../include/eqfield.h"

namespace eqf {

struct WallDev {  // one trap whose walls carry values, Robin loads or channels
  int trap;       // finest-level geometry index
  int rim0;       // first slot of this trap in the rim arrays
  int kind[4];    // EQF_BC_* by EQF_SIDE_*
  double value[4];
  double robs[4];         // dt * rate * s of Robin walls (their load), else 0
  const double* chan[2];  // channel concentrations of the bottom / top walls (or null)
  const double* well;     // the trap's boundary-well concentration (EQF_BC_WELL walls)
};

// Rim of an (nx+1) x (ny+1) lattice, nx, ny >= 3: rows 0, 1, ny-1, ny whole, then
// columns 0, 1, nx-1, nx of rows 2 .. ny-2.
EQF_HD int rim_count(int nx, int ny) { return 4 * (nx + 1) + 4 * (ny - 3); }
EQF_HD void rim_node(int r, int nx, int ny, int& i, int& j) {
  const int band = 4 * (nx + 1);
  if (r < band) {
    const int a = r / (nx + 1);
    i = a < 2 ? a : ny - 3 + a;
    j = r - a * (nx + 1);
  } else {
    const int q = r - band;
    const int b = q & 3;
    i = 2 + (q >> 2);
    j = b < 2 ? b : nx - 3 + b;
  }
}

// Value of Dirichlet node (i, j); bottom and top walls win at the corners.
__device__ __forceinline__ double side_value(const WallDev& w, int side, int j) {
  const int k = w.kind[side];
  if (k == EQF_BC_CHANNEL) return w.chan[side][j];
  if (k == EQF_BC_WELL) return *w.well;
  return w.value[side];
}
__device__ __forceinline__ double wall_value(const WallDev& w, const LevelGeom& g, int i, int j) {
  if (i == 0 && (g.walls & WALL_BOTTOM)) return side_value(w, EQF_SIDE_BOTTOM, j);
  if (i == g.ny && (g.walls & WALL_TOP)) return side_value(w, EQF_SIDE_TOP, j);
  if (j == 0 && (g.walls & WALL_LEFT)) return side_value(w, EQF_SIDE_LEFT, j);
  return side_value(w, EQF_SIDE_RIGHT, j);
}

// F on the rim of every wall trap (blockIdx.y = trap): MODE 0 zeroes it (before the
// point-cell load is summed), MODE 1 copies it into fbase (after), MODE 2 writes
// fbase + the Robin load - the lifting, and the values on Dirichlet rows.
template <int MODE>
__global__ void k_wall_rim(const WallDev* __restrict__ walls, const LevelGeom* __restrict__ G,
                           double* __restrict__ F, double* __restrict__ fbase) {
  const WallDev& w = walls[blockIdx.y];
  const LevelGeom& g = G[w.trap];
  const int nr = rim_count(g.nx, g.ny);
  for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < nr; r += gridDim.x * blockDim.x) {
    int i, j;
    rim_node(r, g.nx, g.ny, i, j);
    const long long k = g.off + (long long)i * g.P + j;
    if (MODE == 0) {
      F[k] = 0.0;
      continue;
    }
    if (MODE == 1) {
      fbase[w.rim0 + r] = F[k];
      continue;
    }
    if (g.walls && is_dirichlet(g, i, j)) {
      F[k] = wall_value(w, g, i, j);
      continue;
    }
    double f = fbase[w.rim0 + r];
    const double hxl = j > 0 ? (j == g.nx ? g.hxl : g.hx) : 0.0;
    const double hxr = j < g.nx ? (j == g.nx - 1 ? g.hxl : g.hx) : 0.0;
    const double hyd = i > 0 ? (i == g.ny ? g.hyl : g.hy) : 0.0;
    const double hyu = i < g.ny ? (i == g.ny - 1 ? g.hyl : g.hy) : 0.0;
    if (i == 0) f += w.robs[EQF_SIDE_BOTTOM] * (hxl + hxr) * 0.5;
    if (i == g.ny) f += w.robs[EQF_SIDE_TOP] * (hxl + hxr) * 0.5;
    if (j == 0) f += w.robs[EQF_SIDE_LEFT] * (hyd + hyu) * 0.5;
    if (j == g.nx) f += w.robs[EQF_SIDE_RIGHT] * (hyd + hyu) * 0.5;
    if (g.walls) {
      LevelGeom q = g;
      q.walls = 0;  // the full operator row
      const Sten<double> s = stencil_general<double>(q, i, j);
      auto lift = [&](int ii, int jj, double c) {
        if (ii >= 0 && ii <= g.ny && jj >= 0 && jj <= g.nx && is_dirichlet(g, ii, jj))
          f -= c * wall_value(w, g, ii, jj);
      };
      lift(i, j + 1, s.e);
      lift(i, j - 1, s.w);
      lift(i + 1, j, s.n);
      lift(i - 1, j, s.s);
      lift(i + 1, j + 1, s.ne);
      lift(i - 1, j - 1, s.sw);
    }
    F[k] = f;
  }
}

struct ChanDev {  // the channels of one trap
  int trap;       // finest-level geometry index
  int n, levels, substeps;
  double h;       // spacing of the flux gradient (the trap's row spacing, 1/npm)
  double dtD;     // dt * D of the trap
  double well;    // well_scaling
  const double* k1;   // PCR multipliers [level * n + i]
  const double* k2;
  const double* bfin;  // 1 / the diagonal after the last level
  const double* bl;    // explicit part: sub-, main and super-diagonal of the right side
  const double* bd;
  const double* bu;
  double* c[2];  // bottom / top concentrations (null: that wall has no channel)
};

constexpr int kChanThreads = 512;
constexpr int kChanMaxNodes = 4097;
__host__ __device__ constexpr size_t chan_smem_bytes(int n) { return (size_t)4 * n * sizeof(double); }

// One reduction sweep of a sub-step, NPT nodes per thread (i = t + q*blockDim): the
// multipliers of level lv+PD are loaded while level lv is reduced, so their L2
// latency is paid once per sweep instead of once per level.  NPT = 0: the plain loop.
// (FP64 throughput bounds the sweep on this part: two FP64 lanes per clock per SM.)
template <int NPT>
__device__ __forceinline__ double* chan_reduce(const ChanDev& ch, double* a, double* b) {
  const int n = ch.n;
  if (NPT == 0) {
    for (int lv = 0, s = 1; lv < ch.levels; ++lv, s <<= 1) {
      const double* K1 = ch.k1 + (size_t)lv * n;
      const double* K2 = ch.k2 + (size_t)lv * n;
      for (int i = threadIdx.x; i < n; i += blockDim.x) {
        double v = a[i];
        if (i - s >= 0) v -= K1[i] * a[i - s];
        if (i + s < n) v -= K2[i] * a[i + s];
        b[i] = v;
      }
      __syncthreads();
      double* t = a;
      a = b;
      b = t;
    }
    return a;
  }
  constexpr int PD = 4, MAXLV = 13;
  double r1[PD][NPT > 0 ? NPT : 1], r2[PD][NPT > 0 ? NPT : 1];
#pragma unroll
  for (int p = 0; p < PD; ++p)
#pragma unroll
    for (int q = 0; q < NPT; ++q) {
      const int i = threadIdx.x + q * blockDim.x;
      const bool ok = p < ch.levels && i < n;
      r1[p][q] = ok ? ch.k1[(size_t)p * n + i] : 0.0;
      r2[p][q] = ok ? ch.k2[(size_t)p * n + i] : 0.0;
    }
#pragma unroll
  for (int lv = 0; lv < MAXLV; ++lv) {
    if (lv >= ch.levels) break;
    const int s = 1 << lv;
    const int slot = lv % PD;
#pragma unroll
    for (int q = 0; q < NPT; ++q) {
      const int i = threadIdx.x + q * blockDim.x;
      if (i < n) {
        double v = a[i];
        if (i - s >= 0) v -= r1[slot][q] * a[i - s];
        if (i + s < n) v -= r2[slot][q] * a[i + s];
        b[i] = v;
      }
      const int nl = lv + PD;  // refill this slot with level lv + PD
      const bool ok = nl < ch.levels && i < n;
      r1[slot][q] = ok ? ch.k1[(size_t)nl * n + i] : 0.0;
      r2[slot][q] = ok ? ch.k2[(size_t)nl * n + i] : 0.0;
    }
    __syncthreads();
    double* t = a;
    a = b;
    b = t;
  }
  return a;
}

// One channel (blockIdx.x = trap, blockIdx.y = 0 bottom / 1 top) through one step:
// the flux of the new trap field u, then `substeps` Crank-Nicolson sub-steps.
template <int NPT>
__global__ void __launch_bounds__(kChanThreads)
    k_channel_step(const ChanDev* __restrict__ chans, const LevelGeom* __restrict__ G,
                   const double* __restrict__ U, const int* __restrict__ frozen) {
  const ChanDev& ch = chans[blockIdx.x];
  double* c = ch.c[blockIdx.y];
  if (!c) return;
  const LevelGeom& g = G[ch.trap];
  if (frozen && frozen[g.trap]) return;
  extern __shared__ __align__(16) unsigned char chan_smem[];
  const int n = ch.n;
  double* flux = reinterpret_cast<double*>(chan_smem);
  double* cc = flux + n;
  double* d0 = cc + n;
  double* d1 = d0 + n;
  const double* u = U + g.off;
  const int P = g.P;
  const int r0 = blockIdx.y == 0 ? 0 : g.ny, r1 = blockIdx.y == 0 ? 1 : g.ny - 1;
  // computeBoundaryFlux: gradc = (u[row next to the wall] - u[wall row]) / h;
  // flux = ds * (dt * D * gradc) / wellScaling with ds = h
  // each sub-step adds flux / substeps: the same share every time, formed once
  const double parts = (double)ch.substeps;
  for (int j = threadIdx.x; j < n; j += blockDim.x) {
    const double gradc = (u[(long long)r1 * P + j] - u[(long long)r0 * P + j]) / ch.h;
    flux[j] = ch.h * (ch.dtD * gradc) / ch.well / parts;
    cc[j] = c[j];
  }
  __syncthreads();
  for (int sub = 0; sub < ch.substeps; ++sub) {
    for (int j = threadIdx.x; j < n; j += blockDim.x) cc[j] += flux[j];
    __syncthreads();
    for (int j = threadIdx.x; j < n; j += blockDim.x) {
      double v = ch.bd[j] * cc[j];
      if (j > 0) v += ch.bl[j] * cc[j - 1];
      if (j < n - 1) v += ch.bu[j] * cc[j + 1];
      d0[j] = v;
    }
    __syncthreads();
    const double* a = chan_reduce<NPT>(ch, d0, d1);
    for (int j = threadIdx.x; j < n; j += blockDim.x) cc[j] = a[j] * ch.bfin[j];
    __syncthreads();
  }
  for (int j = threadIdx.x; j < n; j += blockDim.x) c[j] = cc[j];
}

// --- the boundary well -------------------------------------------------------

struct WellDev {
  int trap;           // finest-level geometry index
  double scale;       // well_scaling
  double decay_dt;    // dt * decay_rate
  double Ddt;         // D * dt of the trap
  double* conc;       // the well concentration
  long long* under;   // underflow count
};

// One block per well trap: the boundary-flux functional -int grad u . n ds of the new
// field (each boundary edge with the gradient of the triangle it bounds, as the
// flux readout), then Simulation::computeBoundaryWell.
__global__ void k_well_update(const WellDev* __restrict__ wells, const LevelGeom* __restrict__ G,
                              const double* __restrict__ U, const int* __restrict__ frozen) {
  const WellDev& w = wells[blockIdx.x];
  const LevelGeom& g = G[w.trap];
  if (frozen && frozen[g.trap]) return;
  const double* u = U + g.off;
  const int P = g.P, nx = g.nx, ny = g.ny;
  double acc = 0.0;
  for (int e = threadIdx.x; e < 2 * (nx + ny); e += blockDim.x) {
    if (e < nx) {  // bottom edge (0, j)-(0, j+1)
      const int k = e;
      acc += (u[k + P + 1] - u[k + 1]) / g.hy * g.hx;
    } else if (e < 2 * nx) {  // top edge (ny, j)-(ny, j+1)
      const int k = (e - nx) + ny * P;
      acc += -(u[k] - u[k - P]) / g.hy * g.hx;
    } else if (e < 2 * nx + ny) {  // left edge (i, 0)-(i+1, 0)
      const int k = (e - 2 * nx) * P;
      acc += (u[k + P + 1] - u[k + P]) / g.hx * g.hy;
    } else {  // right edge (i, nx)-(i+1, nx)
      const int k = (e - 2 * nx - ny) * P + nx;
      acc += -(u[k] - u[k - 1]) / g.hx * g.hy;
    }
  }
  const double total = block_sum(acc);
  if (threadIdx.x == 0) {
    const double flux = w.Ddt * total;  // totalBoundaryFlux
    double c = *w.conc;
    c += flux / w.scale;
    c -= w.decay_dt * c;
    if (c < 0.0) {
      c = 0.0;
      *w.under += 1;
    }
    *w.conc = c;
  }
}

}  // namespace eqf
