// Cell <-> node transfer kernels.
//
// Deposit (cell -> node): each point cell i of a trap loads dt * s_i * phi_j(x_i)
// onto the three vertices j of its containing triangle.  The three (node, weight)
// entries of every cell are sorted by node with a counting sort whose buckets are
// then ordered by entry index, so each node sums its contributions in one fixed
// order: the load is bit-identical whatever the batch composition or launch
// timing (no floating-point atomics).  The reference deposits onto interior lattice
// nodes of rod cells instead (src/abm/eQabm.cpp:338-359); the point-cell load is
// the workload's source model.
//
// Gather (node -> cell): c(x_i) = sum_j phi_j(x_i) c_j on the same triangle.
#pragma once
#include "eqf_common.cuh"

namespace eqf {

struct CellGeom {  // per trap: fine-level mesh for locating cells
  long long off;
  int nx, ny, P;  // cells along x / y, device row pitch
  double hx, hy;
};

// Containing triangle and barycentric weights of (x, y) on a trap's fine mesh.
// Points on the square diagonal belong to the lower-right triangle (v0, v1, v3).
__device__ __forceinline__ void locate(const CellGeom& g, double x, double y, int node[3],
                                       double wgt[3]) {
  const double X = x / g.hx, Y = y / g.hy;
  int j = (int)floor(X), i = (int)floor(Y);
  j = j < 0 ? 0 : (j > g.nx - 1 ? g.nx - 1 : j);
  i = i < 0 ? 0 : (i > g.ny - 1 ? g.ny - 1 : i);
  const double xi = X - j, eta = Y - i;
  const int v0 = j + i * g.P;
  node[0] = v0;
  node[2] = v0 + g.P + 1;
  if (xi >= eta) {
    node[1] = v0 + 1;
    wgt[0] = 1.0 - xi;
    wgt[1] = xi - eta;
    wgt[2] = eta;
  } else {
    node[1] = v0 + g.P;
    wgt[0] = 1.0 - eta;
    wgt[1] = eta - xi;
    wgt[2] = xi;
  }
}

// entries 3c..3c+2 of cell c: global fine node index and weight; counts[node]++
__global__ void k_cells_locate(int ncells, const CellGeom* __restrict__ cg,
                               const int* __restrict__ cell_trap,
                               const double* __restrict__ cell_xy, int* __restrict__ ent_node,
                               double* __restrict__ ent_w, int* __restrict__ counts) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= ncells) return;
  const CellGeom g = cg[cell_trap[c]];
  int node[3];
  double w[3];
  locate(g, cell_xy[2 * c], cell_xy[2 * c + 1], node, w);
  for (int v = 0; v < 3; ++v) {
    const int gn = (int)(g.off + node[v]);
    ent_node[3 * c + v] = gn;
    ent_w[3 * c + v] = w[v];
    atomicAdd(&counts[gn], 1);  // integer: the final counts are exact
  }
}

// pos = start[node] + arrival rank (arrival order is not deterministic; fixed below)
__global__ void k_cells_place(int nent, const int* __restrict__ ent_node,
                              const int* __restrict__ start, int* __restrict__ cursor,
                              int* __restrict__ perm) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= nent) return;
  const int n = ent_node[e];
  perm[start[n] + atomicAdd(&cursor[n], 1)] = e;
}

// head[p] = 1 where a node's bucket starts in the sorted order (read-only pass).
__global__ void k_cells_heads(int nent, const int* __restrict__ ent_node,
                              const int* __restrict__ start, const int* __restrict__ perm,
                              int* __restrict__ head) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= nent) return;
  head[p] = start[ent_node[perm[p]]] == p ? 1 : 0;
}

// Canonical order of each segment (the entries of one node): by the contributing
// cell's (x, y, rate), or by the value for explicit nodal increments, then by entry
// index.  The summation order then depends only on the set of contributions, so
// the deposit is bit-identical under any permutation of the cells.  One thread per
// segment; segments hold a handful of entries.
__device__ __forceinline__ bool entry_less(int e1, int e2, const double* __restrict__ xy,
                                           const double* __restrict__ s,
                                           const double* __restrict__ val) {
  if (xy) {
    const int c1 = e1 / 3, c2 = e2 / 3;
    if (xy[2 * c1] != xy[2 * c2]) return xy[2 * c1] < xy[2 * c2];
    if (xy[2 * c1 + 1] != xy[2 * c2 + 1]) return xy[2 * c1 + 1] < xy[2 * c2 + 1];
    if (s[c1] != s[c2]) return s[c1] < s[c2];
  } else if (val[e1] != val[e2]) {
    return val[e1] < val[e2];
  }
  return e1 < e2;
}

__global__ void k_seg_sort(int nseg, const int* __restrict__ seg_start, int* __restrict__ perm,
                           const double* __restrict__ xy, const double* __restrict__ s,
                           const double* __restrict__ val) {
  const int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= nseg) return;
  const int a = seg_start[q], b = seg_start[q + 1];
  for (int i = a + 1; i < b; ++i) {
    const int v = perm[i];
    int j = i - 1;
    while (j >= a && entry_less(v, perm[j], xy, s, val)) {
      perm[j + 1] = perm[j];
      --j;
    }
    perm[j + 1] = v;
  }
}

// seg_start[s] = sorted position of segment s's first entry (from the scanned heads)
__global__ void k_cells_segments(int nent, const int* __restrict__ head,
                                 const int* __restrict__ head_scan, int* __restrict__ seg_start,
                                 int nseg) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p < nent && head[p]) seg_start[head_scan[p]] = p;
  if (p == 0) seg_start[nseg] = nent;
}

// out[node] (=, or += when ADD) sum of ent_val over the node's entries, in entry order
template <bool ADD>
__global__ void k_seg_sum(int nseg, const int* __restrict__ seg_start, const int* __restrict__ perm,
                          const int* __restrict__ ent_node, const double* __restrict__ ent_val,
                          double* __restrict__ out) {
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= nseg) return;
  const int a = seg_start[s], b = seg_start[s + 1];
  double acc = 0.0;
  for (int p = a; p < b; ++p) acc += ent_val[perm[p]];
  const int node = ent_node[perm[a]];
  if (ADD)
    out[node] += acc;
  else
    out[node] = acc;
}

// ent_val[3c+v] = ent_w[3c+v] * s[c] * scale[trap(c)]
__global__ void k_cells_values(int ncells, const double* __restrict__ ent_w,
                               const double* __restrict__ cell_s, const double* __restrict__ scale,
                               const int* __restrict__ cell_trap, double* __restrict__ ent_val) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= ncells) return;
  const double f = cell_s[c] * scale[cell_trap[c]];
  for (int v = 0; v < 3; ++v) ent_val[3 * c + v] = ent_w[3 * c + v] * f;
}

// entries of explicit nodal increments: ent_node = off[trap] + node; counts[node]++
// node[e] is a grid-order index (row length nx+1); the device rows have pitch P
__global__ void k_nodal_entries(int n, long long off, int row, int P,
                                const long long* __restrict__ node, int* __restrict__ ent_node,
                                int* __restrict__ counts) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= n) return;
  const long long k = node[e];
  const int gn = (int)(off + (k / row) * P + k % row);
  ent_node[e] = gn;
  atomicAdd(&counts[gn], 1);
}

// out[c] = sum_v w_v u[node_v]
__global__ void k_cells_gather(int ncells, const int* __restrict__ ent_node,
                               const double* __restrict__ ent_w, const double* __restrict__ u,
                               double* __restrict__ out) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= ncells) return;
  double acc = 0.0;
  for (int v = 0; v < 3; ++v) acc += ent_w[3 * c + v] * u[ent_node[3 * c + v]];
  out[c] = acc;
}

// Two-species sender/receiver sources from the concentrations gathered at the
// cell centres (cells_c, indexed like the batch cell arrays).  Coupled cell q has
// index i1[q] in species 1's trap and i2[q] in species 2's trap:
//   s1 = sender * prod1 - uptake * c1
//   s2 = (1 - sender) * vmax * c1 / (K + c1) - uptake * c2
struct CouplingLaw {
  double vmax, K, uptake;
};
__global__ void k_cells_qs_sources(int n, const int* __restrict__ i1, const int* __restrict__ i2,
                                   const int* __restrict__ sender,
                                   const double* __restrict__ prod1,
                                   const int* __restrict__ law_of, const CouplingLaw* __restrict__ law,
                                   const double* __restrict__ cells_c, double* __restrict__ rate) {
  const int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= n) return;
  const CouplingLaw L = law[law_of[q]];
  const double c1 = cells_c[i1[q]], c2 = cells_c[i2[q]];
  const int snd = sender[q];
  rate[i1[q]] = (snd ? prod1[q] : 0.0) - L.uptake * c1;
  rate[i2[q]] = (snd ? 0.0 : L.vmax * c1 / (L.K + c1)) - L.uptake * c2;
}

// ---------------------------------------------------------------------------
// Exclusive scan of int32 (deterministic), three phases.
constexpr int kScanBlock = 1024;
constexpr int kScanItems = 4;  // per thread
constexpr int kScanTile = kScanBlock * kScanItems;

__device__ __forceinline__ int block_excl_scan(int v, int& total) {
  __shared__ int ws[32];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  int x = v;
  for (int o = 1; o < 32; o <<= 1) {
    const int y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) ws[w] = x;
  __syncthreads();
  if (w == 0) {
    int s = lane < (int)(blockDim.x >> 5) ? ws[lane] : 0;
    for (int o = 1; o < 32; o <<= 1) {
      const int y = __shfl_up_sync(0xffffffffu, s, o);
      if (lane >= o) s += y;
    }
    ws[lane] = s;
  }
  __syncthreads();
  total = ws[(blockDim.x >> 5) - 1];
  const int pre = w > 0 ? ws[w - 1] : 0;
  __syncthreads();
  return pre + x - v;
}

__global__ void k_scan_sums(int n, const int* __restrict__ in, int* __restrict__ sums) {
  const int base = blockIdx.x * kScanTile + threadIdx.x * kScanItems;
  int v = 0;
  for (int q = 0; q < kScanItems; ++q)
    if (base + q < n) v += in[base + q];
  int total;
  block_excl_scan(v, total);
  if (threadIdx.x == 0) sums[blockIdx.x] = total;
}

// single CTA: exclusive scan of the block sums in place
__global__ void k_scan_top(int nb, int* __restrict__ sums) {
  int carry = 0;
  for (int b0 = 0; b0 < nb; b0 += blockDim.x) {
    const int idx = b0 + threadIdx.x;
    const int v = idx < nb ? sums[idx] : 0;
    int total;
    const int ex = block_excl_scan(v, total);
    if (idx < nb) sums[idx] = carry + ex;
    carry += total;
    __syncthreads();
  }
}

// out[i] = exclusive prefix; out[n] = total
__global__ void k_scan_apply(int n, const int* __restrict__ in, const int* __restrict__ sums,
                             int* __restrict__ out) {
  const int base = blockIdx.x * kScanTile + threadIdx.x * kScanItems;
  int vals[kScanItems];
  int v = 0;
  for (int q = 0; q < kScanItems; ++q) {
    vals[q] = base + q < n ? in[base + q] : 0;
    v += vals[q];
  }
  int total;
  int ex = block_excl_scan(v, total) + sums[blockIdx.x];
  for (int q = 0; q < kScanItems; ++q) {
    if (base + q < n) out[base + q] = ex;
    ex += vals[q];
    if (base + q == n - 1) out[n] = ex;
  }
}

}  // namespace eqf
