// Rod cells of the agent-based model coupled to the field the reference's way.
//
// Per cell (src/abm/eQabm.cpp:234-390):
//   footprint  the lattice nodes strictly inside the cell's first body half, searched
//              over the pole bounding box widened by nodesToEdge (findInteriorPoints,
//              eQabm.cpp:268-304; cpmEcoli::pointIsInCell, cpmEcoli.cpp:313-328), or
//              the centre node when none is inside;
//   gather     eHSL = mean of the field over the footprint, summed in footprint order
//              (readHSL, eQabm.cpp:326-337);
//   exchange   dHSL = dt*k_m*(iHSL - eHSL) in nM and the intracellular update
//              (Strain::computeConcentrations / pushConcentrations, src/Strain.h:281-345;
//              sendRecvStrain::computeProteins, src/Strain.cpp:10-73);
//   deposit    dHSL converted to molecules, to the extracellular volume and to one
//              lattice node, split equally over the footprint and added to the field
//              (writeHSL, eQabm.cpp:338-359; eQ::Cell, src/eQcell.h:42-97).
//
// The reference runs the cells one after the other, so a cell reads what earlier
// cells deposited on shared nodes.  Here the cells are grouped into waves: a cell's
// wave is one more than the latest wave of any earlier cell sharing a node with it,
// so within a wave no two cells touch the same node and every node sees its
// deposits in cell order.  Each wave is one launch over every rod set of the
// batch, one thread per cell.
//
// Every floating-point operation is a separately rounded IEEE operation (no fused
// multiply-add), in the reference's order, so results match the reference's
// double-precision arithmetic bit for bit.
#pragma once
#include "eqf_common.cuh"
#include "../../include/eqfield.h"

namespace eqf {

constexpr int kRodLayers = EQF_MAX_ROD_LAYERS;

// eQ::Cell constants (src/eQcell.h:42-59), evaluated in the reference's order:
// poleRadius = W/2, cylindrical volume per length = pi*r*r, both poles 4/3*pi*r^3,
// nanoMolarPerMoleculePerCubicMicron = 1/0.602.
struct RodConst {
  double cyl, pole, nm_per_molecule;
};

struct RodLawDev {  // one rod set
  double npm, dt;
  double km[kRodLayers];
  long long lay_off[kRodLayers];  // fine-level field offset of each layer's trap
  int trap0;                      // first layer's trap (frozen traps skip the exchange)
  int nlayers;
  int nx, ny, P;  // lattice (ny+1) x (nx+1) nodes, device row pitch P
  int nte;        // nodesToEdge = round(npm * W/2) (eQabm.cpp:75)
  RodConst k;
};

__device__ __forceinline__ double r_mul(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ double r_add(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ double r_sub(double a, double b) { return __dsub_rn(a, b); }
__device__ __forceinline__ double r_div(double a, double b) { return __ddiv_rn(a, b); }

// C's round() for x >= 0 (half away from zero): the lattice index of eQ::data::ij_from_xy
// (src/eQ.h:118-123); inputs are validated non-negative on the host.
__device__ __forceinline__ int r_round(double x) {
  const double f = floor(x);
  return (int)f + (r_sub(x, f) >= 0.5 ? 1 : 0);
}

struct RodBox {
  int i1, i2, j1, j2;
};

// Search rectangle of eQabm.cpp:276-287 (i: row / y, j: column / x).
__device__ __forceinline__ RodBox rod_box(const eqf_rod& r, const RodLawDev& L) {
  const int ai = r_round(r_mul(r.pole_a[1], L.npm)), aj = r_round(r_mul(r.pole_a[0], L.npm));
  const int bi = r_round(r_mul(r.pole_b[1], L.npm)), bj = r_round(r_mul(r.pole_b[0], L.npm));
  RodBox b;
  b.i1 = ai > bi ? bi : ai;
  b.i2 = ai > bi ? ai : bi;
  b.j1 = aj > bj ? bj : aj;
  b.j2 = aj > bj ? aj : bj;
  b.i1 = b.i1 >= L.nte ? b.i1 - L.nte : 0;
  b.j1 = b.j1 >= L.nte ? b.j1 - L.nte : 0;
  b.i2 = b.i2 + L.nte >= L.ny ? L.ny : b.i2 + L.nte;  // nodesHigh - 1 = ny
  b.j2 = b.j2 + L.nte >= L.nx ? L.nx : b.j2 + L.nte;  // nodesWide - 1 = nx
  // poles inside the trap give i1 <= ny, j1 <= nx; the clamps only guard memory
  b.i1 = min(b.i1, L.ny);
  b.j1 = min(b.j1, L.nx);
  return b;
}

// The cell's first body half: world -> local transform and its box edges.
// World -> local is chipmunk 7.0.1's cpBodyWorldToLocal (the rigid inverse of the
// body transform [c -s px; s c py] applied to the point; the body's centre of
// gravity is its position, as eQ never gives its shapes mass).
struct RodFrame {
  double c, s, tx, ty;  // local = (c*x + s*y + tx, -s*x + c*y + ty)
  double v[8], e[8];
};

__device__ __forceinline__ RodFrame rod_frame(const eqf_rod& r) {
  RodFrame f;
  f.c = r.body_rot[0];
  f.s = r.body_rot[1];
  const double px = r.body_pos[0], py = r.body_pos[1];
  f.tx = r_sub(r_mul(-f.s, py), r_mul(px, f.c));
  f.ty = r_sub(r_mul(px, f.s), r_mul(f.c, py));
#pragma unroll
  for (int q = 0; q < 8; ++q) f.v[q] = r.verts[q];
  // cpmEcoli::computeCellBoudaryEdges (cpmEcoli.cpp:71-76): edge k = v[k+1] - v[k]
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    const int n = (k + 1) & 3;
    f.e[2 * k] = r_sub(f.v[2 * n], f.v[2 * k]);
    f.e[2 * k + 1] = r_sub(f.v[2 * n + 1], f.v[2 * k + 1]);
  }
  return f;
}

// pointIsInCell: all four cross(edge_k, p - v_{k+1}) strictly negative.
__device__ __forceinline__ bool rod_inside(const RodFrame& f, double x, double y) {
  const double lx = r_add(r_add(r_mul(f.c, x), r_mul(f.s, y)), f.tx);
  const double ly = r_add(r_add(r_mul(-f.s, x), r_mul(f.c, y)), f.ty);
  bool in = true;
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    const int n = (k + 1) & 3;
    const double px = r_sub(lx, f.v[2 * n]), py = r_sub(ly, f.v[2 * n + 1]);
    const double cr = r_sub(r_mul(f.e[2 * k], py), r_mul(f.e[2 * k + 1], px));
    in = in && (cr < 0.0);
  }
  return in;
}

// Footprint of every cell, one warp per cell.  COUNT: count[c] = footprint size.
// FILL: node[off[c] ..] = the footprint's lattice nodes (i*P + j, relative to the
// trap) in the reference's search order (rows i ascending, then columns j), and
// ent_cell[...] = c.
template <bool FILL>
__global__ void k_rod_footprint(int n, const eqf_rod* __restrict__ rods,
                                const RodLawDev* __restrict__ law, int* __restrict__ count,
                                const int* __restrict__ off, int* __restrict__ node,
                                int* __restrict__ ent_cell) {
  const int lane = threadIdx.x & 31;
  const int warps = (gridDim.x * blockDim.x) >> 5;
  const RodLawDev L = *law;
  for (int c = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; c < n; c += warps) {
    const eqf_rod& r = rods[c];
    const RodBox b = rod_box(r, L);
    const RodFrame f = rod_frame(r);
    const int bw = b.j2 - b.j1 + 1;
    const long long total = (long long)bw * (b.i2 - b.i1 + 1);
    const int base = FILL ? off[c] : 0;
    int k = 0;
    for (long long q0 = 0; q0 < total; q0 += 32) {
      const long long q = q0 + lane;
      bool in = false;
      int i = 0, j = 0;
      if (q < total) {
        i = b.i1 + (int)(q / bw);
        j = b.j1 + (int)(q % bw);
        // eQ::data::xy_from_ij (src/eQ.h:114-117)
        in = rod_inside(f, r_div((double)j, L.npm), r_div((double)i, L.npm));
      }
      const unsigned m = __ballot_sync(0xffffffffu, in);
      if (FILL && in) {
        const int p = base + k + __popc(m & ((1u << lane) - 1u));
        node[p] = i * L.P + j;
        ent_cell[p] = c;
      }
      k += __popc(m);
    }
    if (k == 0) {  // no interior node: the centre node (eQabm.cpp:299-303)
      if (FILL && lane == 0) {
        // the host keeps centres inside the trap and W*npm = nx, H*npm = ny, so
        // these rounded indices lie on the lattice; the clamps only guard memory
        const int i = min(r_round(r_mul(r.center[1], L.npm)), L.ny);
        const int j = min(r_round(r_mul(r.center[0], L.npm)), L.nx);
        node[base] = i * L.P + j;
        ent_cell[base] = c;
      }
      k = 1;
    }
    if (!FILL && lane == 0) count[c] = k;
  }
}

// --- dependency waves (only when some node lies in two footprints) ----------

// cover[key]++ per footprint entry (key = node + the set's key base); *shared = 1
// if a node is covered twice.
__global__ void k_rod_cover(int nent, const int* __restrict__ node, long long key0,
                            int* __restrict__ cover, int* __restrict__ shared) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= nent) return;
  if (atomicAdd(&cover[key0 + node[e]], 1) > 0) *shared = 1;
}

// Entries bucketed by node: pos = start[node] + arrival rank.
__global__ void k_rod_place(int nent, const int* __restrict__ node, long long key0,
                            const int* __restrict__ start, int* __restrict__ cursor,
                            int* __restrict__ perm) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= nent) return;
  const long long key = key0 + node[e];
  perm[start[key] + atomicAdd(&cursor[key], 1)] = e;
}

// Each bucket ordered by cell (= entry index: entries are cell-major), by the thread
// at the bucket's first position; then pred[p] = the cell before position p in its
// bucket (-1 at a bucket head).
__global__ void k_rod_bucket_order(int nent, const int* __restrict__ node, long long key0,
                                   const int* __restrict__ start,
                                   const int* __restrict__ cover, int* __restrict__ perm) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= nent) return;
  const long long key = key0 + node[perm[p]];
  if (start[key] != p) return;
  const int a = p, b = p + cover[key];
  for (int i = a + 1; i < b; ++i) {
    const int v = perm[i];
    int j = i - 1;
    while (j >= a && perm[j] > v) {
      perm[j + 1] = perm[j];
      --j;
    }
    perm[j + 1] = v;
  }
}

__global__ void k_rod_preds(int nent, const int* __restrict__ node, long long key0,
                            const int* __restrict__ start, const int* __restrict__ perm,
                            const int* __restrict__ ent_cell, int* __restrict__ pred,
                            int* __restrict__ succ) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= nent) return;
  const long long key = key0 + node[perm[p]];
  succ[p] = ent_cell[perm[p]];
  pred[p] = start[key] == p ? -1 : ent_cell[perm[p - 1]];
}

// The waves of one rod set in one CTA: passes of wave[c] = max over c's predecessors
// of wave[pred] + 1, separated by CTA barriers, until a pass changes nothing.  A chain of n cells settles within n
// passes; past that bound the kernel stops and sets *unsettled (never expected).
// *passes receives the number of passes run (the last one changing nothing): each
// costs one sweep over all nent entries on this one CTA, so the relaxation's time
// grows with nent times the longest dependency chain.
__global__ void __launch_bounds__(1024)
    k_rod_relax_all(int nent, int n, const int* __restrict__ pred, const int* __restrict__ succ,
                    int* __restrict__ wave, int* __restrict__ unsettled,
                    int* __restrict__ passes) {
  __shared__ int changed;
  for (int pass = 0; pass <= n + 1; ++pass) {
    if (threadIdx.x == 0) changed = 0;
    __syncthreads();
    for (int p = threadIdx.x; p < nent; p += blockDim.x) {
      const int a = pred[p];
      if (a < 0) continue;
      // L2 reads: the other threads' updates are atomics performed there
      const int w = __ldcg(&wave[a]) + 1;
      const int c = succ[p];
      if (w > __ldcg(&wave[c]) && atomicMax(&wave[c], w) < w) changed = 1;
    }
    __syncthreads();  // this pass's waves are visible to the whole CTA
    if (!changed) {
      if (threadIdx.x == 0) *passes = pass + 1;
      return;
    }
    __syncthreads();  // every thread has read `changed` before it is reset
  }
  if (threadIdx.x == 0) {
    *unsettled = 1;
    *passes = n + 2;
  }
}

// wave sizes and the highest wave
__global__ void k_rod_wave_count(int n, const int* __restrict__ wave, int* __restrict__ wcount,
                                 int* __restrict__ wmax) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= n) return;
  atomicAdd(&wcount[wave[c]], 1);
  atomicMax(wmax, wave[c]);
}

// cells grouped by wave (order within a wave is free: its cells are independent)
__global__ void k_rod_wave_place(int n, const int* __restrict__ wave,
                                 const int* __restrict__ wstart, int* __restrict__ wcursor,
                                 int* __restrict__ cells) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= n) return;
  cells[wstart[wave[c]] + atomicAdd(&wcursor[wave[c]], 1)] = c;
}

__global__ void k_rod_iota(int n, int* __restrict__ cells) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c < n) cells[c] = c;
}

// Per cell in wave order: (cell, footprint offset, footprint size), and per cell
// the eQ::Cell volume constants of its length, evaluated as the reference does:
// computeCellVolumeActual V = (L - W) * pi r^2 + 4/3 pi r^3,
// moleculeNumberToNanoMolar(1, L) = (1/V) * nM-per-molecule-per-um^3 and
// computeExtraCellularVolumeFraction = 1 - V / (L*1*1) (src/eQcell.h:61-93).
__global__ void k_rod_cell_info(int n, const int* __restrict__ cells,
                                const int* __restrict__ fp_off, const eqf_rod* __restrict__ rods,
                                const RodLawDev* __restrict__ law, int4* __restrict__ winfo,
                                double* __restrict__ cellk) {
  const int idx = blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= n) return;
  const int c = cells[idx];
  winfo[idx] = make_int4(c, fp_off[c], fp_off[c + 1] - fp_off[c], 0);
  const RodConst k = law->k;
  const double len = rods[c].length;
  const double V = r_add(r_mul(r_sub(len, 1.0), k.cyl), k.pole);
  cellk[3 * c] = V;
  cellk[3 * c + 1] = r_mul(r_div(1.0, V), k.nm_per_molecule);
  cellk[3 * c + 2] = r_sub(1.0, r_div(V, len));
}

// --- the per-step exchange ---------------------------------------------------

// What one wave launch needs of a rod set (device copy; the launch indexes it by
// blockIdx.y, so pointer changes never invalidate a captured step).
struct RodSetDev {
  const int* woff;    // woff[w] .. woff[w+1]: cells of wave w
  const int4* winfo;  // in wave order: (cell, footprint offset, footprint size, 0)
  const double* cellk;  // per cell: volume, nM per molecule, extracellular fraction
  const eqf_rod* rods;
  const RodLawDev* law;
  const int* fp_node;  // lattice nodes relative to the trap
  double* ihsl;        // per cell and layer [c*kRodLayers + l]: molecules
  const double* prod;  // nM per time unit
  const unsigned char* mode;  // EQF_ROD_*
  double* ehsl;        // out: the gathered footprint mean
  int waves;
};

// The exchange of one cell once its footprint sums are known: the gathered means,
// the membrane exchange and intracellular update, and the per-node deposit d[l]
// (dep[l] false: the layer takes no deposit).
template <int NL>
__device__ __forceinline__ void rod_exchange_values(const RodSetDev& S, const RodLawDev& L,
                                                    int c, int K, const double* sum,
                                                    double* d, bool* dep) {
  // per-cell volume constants (k_rod_cell_info)
  const double V = S.cellk[3 * c], nmpm = S.cellk[3 * c + 1], ecf = S.cellk[3 * c + 2];
  const double Kd = (double)K;
#pragma unroll
  for (int l = 0; l < NL; ++l) {
    // readHSL: the footprint sum over the point count
    const double e = r_div(sum[l], Kd);
    const int s = c * kRodLayers + l;
    const int md = S.mode[s];
    S.ehsl[s] = e;
    dep[l] = md != EQF_ROD_INERT;
    d[l] = 0.0;
    if (!dep[l]) continue;
    // computeConcentrations: iHSL *= nanoMolarPerMolecule; dHSL = dt*(k_m*(iHSL - eHSL))
    const double inm = r_mul(S.ihsl[s], nmpm);
    const double dH = r_mul(L.dt, r_mul(L.km[l], r_sub(inm, e)));
    // computeProteins: deltaHSL = dt*alpha - dHSL (circuit) or 0 (held)
    const double delta = md == EQF_ROD_CIRCUIT ? r_sub(r_mul(L.dt, S.prod[s]), dH) : 0.0;
    // pushConcentrations: iHSL += deltaHSL, clamped at 0, stored as molecules
    double inew = r_add(inm, delta);
    if (inew < 0.0) inew = 0.0;
    S.ihsl[s] = r_div(inew, nmpm);
    // writeHSL: molecules / extracellular fraction * npm^2 / K on every node
    const double number = r_mul(r_div(dH, L.k.nm_per_molecule), V);
    const double per_um2 = r_div(number, ecf);
    d[l] = r_div(r_mul(r_mul(per_um2, L.npm), L.npm), Kd);
  }
}

// One cell of a wave, NL layers.  The layers share the footprint walk and the
// node loads are issued B at a time (the sums stay in footprint order).
template <int NL, int B>
__device__ __forceinline__ void rod_cell(const RodSetDev& S, const RodLawDev& L, int c, int f0,
                                         int K, double* __restrict__ U) {
  const int* __restrict__ fp = S.fp_node + f0;
  double* u[NL];
#pragma unroll
  for (int l = 0; l < NL; ++l) u[l] = U + L.lay_off[l];
  double sum[NL], d[NL];
  bool dep[NL];
#pragma unroll
  for (int l = 0; l < NL; ++l) sum[l] = 0.0;
  int k = 0;
  for (; k + B <= K; k += B) {
    int n[B];
    double v[NL][B];
#pragma unroll
    for (int q = 0; q < B; ++q) n[q] = fp[k + q];
#pragma unroll
    for (int l = 0; l < NL; ++l)
#pragma unroll
      for (int q = 0; q < B; ++q) v[l][q] = u[l][n[q]];
#pragma unroll
    for (int l = 0; l < NL; ++l)
#pragma unroll
      for (int q = 0; q < B; ++q) sum[l] = r_add(sum[l], v[l][q]);
  }
  if (k < K) {  // the last K - k < B nodes: one predicated round of loads
    int n[B];
    double v[NL][B];
#pragma unroll
    for (int q = 0; q < B; ++q) n[q] = k + q < K ? fp[k + q] : 0;
#pragma unroll
    for (int l = 0; l < NL; ++l)
#pragma unroll
      for (int q = 0; q < B; ++q) v[l][q] = k + q < K ? u[l][n[q]] : 0.0;
#pragma unroll
    for (int l = 0; l < NL; ++l)
#pragma unroll
      for (int q = 0; q < B; ++q)
        if (k + q < K) sum[l] = r_add(sum[l], v[l][q]);
  }
  rod_exchange_values<NL>(S, L, c, K, sum, d, dep);
  // deposit: the footprint's nodes are distinct, so each group of loads may run
  // ahead of the group's stores
  k = 0;
  for (; k + B <= K; k += B) {
    int n[B];
#pragma unroll
    for (int q = 0; q < B; ++q) n[q] = fp[k + q];
#pragma unroll
    for (int l = 0; l < NL; ++l) {
      if (!dep[l]) continue;
      double v[B];
#pragma unroll
      for (int q = 0; q < B; ++q) v[q] = u[l][n[q]];
#pragma unroll
      for (int q = 0; q < B; ++q) u[l][n[q]] = r_add(v[q], d[l]);
    }
  }
  if (k < K) {
    int n[B];
#pragma unroll
    for (int q = 0; q < B; ++q) n[q] = k + q < K ? fp[k + q] : 0;
#pragma unroll
    for (int l = 0; l < NL; ++l) {
      if (!dep[l]) continue;
      double v[B];
#pragma unroll
      for (int q = 0; q < B; ++q) v[q] = k + q < K ? u[l][n[q]] : 0.0;
#pragma unroll
      for (int q = 0; q < B; ++q)
        if (k + q < K) u[l][n[q]] = r_add(v[q], d[l]);
    }
  }
}

// The stashed form for footprints of at most KS nodes: the gather walks the
// footprint in rounds of B loads with the next round's node indices prefetched,
// and keeps every value and index in shared memory (this thread's slice, strided
// by the block size), so the deposit is stores only -- no other cell of the wave
// touches these nodes.
constexpr int kRodStash = 64;     // footprint nodes held per thread
constexpr int kRodThreads = 64;   // threads per block of the exchange

__host__ __device__ constexpr size_t rod_stash_bytes(int nl) {
  return (size_t)kRodThreads * kRodStash * (nl * sizeof(double) + sizeof(int));
}

template <int NL, int B>
__device__ __forceinline__ void rod_cell_stash(const RodSetDev& S, const RodLawDev& L, int c,
                                               int f0, int K, double* __restrict__ U,
                                               double* __restrict__ smv, int* __restrict__ smi) {
  const int t = threadIdx.x, nt = kRodThreads;
  const int* __restrict__ fp = S.fp_node + f0;
  double* u[NL];
#pragma unroll
  for (int l = 0; l < NL; ++l) u[l] = U + L.lay_off[l];
  double sum[NL], d[NL];
  bool dep[NL];
#pragma unroll
  for (int l = 0; l < NL; ++l) sum[l] = 0.0;
  int nn[B];
#pragma unroll
  for (int q = 0; q < B; ++q) nn[q] = q < K ? fp[q] : 0;
  for (int k = 0; k < K; k += B) {
    int cur[B];
    double v[NL][B];
#pragma unroll
    for (int q = 0; q < B; ++q) cur[q] = nn[q];
#pragma unroll
    for (int l = 0; l < NL; ++l)
#pragma unroll
      for (int q = 0; q < B; ++q) v[l][q] = k + q < K ? u[l][cur[q]] : 0.0;
#pragma unroll
    for (int q = 0; q < B; ++q) nn[q] = k + B + q < K ? fp[k + B + q] : 0;
#pragma unroll
    for (int q = 0; q < B; ++q) {
      if (k + q < K) {
        smi[(k + q) * nt + t] = cur[q];
#pragma unroll
        for (int l = 0; l < NL; ++l) {
          sum[l] = r_add(sum[l], v[l][q]);  // footprint order
          smv[(l * kRodStash + k + q) * nt + t] = v[l][q];
        }
      }
    }
  }
  rod_exchange_values<NL>(S, L, c, K, sum, d, dep);
#pragma unroll
  for (int l = 0; l < NL; ++l) {
    if (!dep[l]) continue;
    for (int q = 0; q < K; ++q)
      u[l][smi[q * nt + t]] = r_add(smv[(l * kRodStash + q) * nt + t], d[l]);
  }
}

// One wave of every rod set: one thread per cell (the cells of a wave touch
// disjoint nodes).  A cell's gather is a serial sum in footprint order, so one
// thread per cell lets 32 cells share each double-precision instruction.  NL is
// the batch's largest layer count; a set with fewer layers takes the matching
// instantiation of the cell body.
template <int NL>
__global__ void __launch_bounds__(kRodThreads) k_rod_exchange(
    int wave, const RodSetDev* __restrict__ sets, const int* __restrict__ frozen,
    double* __restrict__ U) {
  extern __shared__ __align__(16) unsigned char rod_smem[];
  double* smv = reinterpret_cast<double*>(rod_smem);
  int* smi = reinterpret_cast<int*>(smv + (size_t)NL * kRodStash * kRodThreads);
  const RodSetDev S = sets[blockIdx.y];  // by value: its loads issue together
  if (wave >= S.waves) return;
  const RodLawDev L = *S.law;
  if (frozen && frozen[L.trap0]) return;
  const int a = S.woff[wave], b = S.woff[wave + 1];
  const int nl = L.nlayers;
  for (int idx = a + blockIdx.x * blockDim.x + threadIdx.x; idx < b;
       idx += gridDim.x * blockDim.x) {
    const int4 w = S.winfo[idx];
    if (w.z <= kRodStash) {
      if (NL == 1 || nl == 1)
        rod_cell_stash<1, 16>(S, L, w.x, w.y, w.z, U, smv, smi);
      else if (NL == 2 || nl == 2)
        rod_cell_stash<2, 16>(S, L, w.x, w.y, w.z, U, smv, smi);
      else if (NL == 3 || nl == 3)
        rod_cell_stash<(NL < 3 ? NL : 3), 8>(S, L, w.x, w.y, w.z, U, smv, smi);
      else
        rod_cell_stash<NL, 8>(S, L, w.x, w.y, w.z, U, smv, smi);
    } else if (NL == 1 || nl == 1) {
      rod_cell<1, 8>(S, L, w.x, w.y, w.z, U);
    } else if (NL == 2 || nl == 2) {
      rod_cell<2, 8>(S, L, w.x, w.y, w.z, U);
    } else if (NL == 3 || nl == 3) {
      rod_cell<(NL < 3 ? NL : 3), 8>(S, L, w.x, w.y, w.z, U);
    } else {
      rod_cell<NL, 8>(S, L, w.x, w.y, w.z, U);
    }
  }
}

}  // namespace eqf
