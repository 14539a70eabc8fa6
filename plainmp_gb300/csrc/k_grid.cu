// Device construction of the point-cloud grid used in place of the reference KD-tree
// (collision/kdtree.cpp:20-65).  Steps: fine-cell key per point (cells numbered
// block-major) -> per-cell counts -> exclusive scan -> scatter -> occupied-cell records with
// conservative FP32 boxes -> per-block record ranges and boxes.  The order of points inside a
// cell follows atomic arrival and is not fixed; nearest distances do not depend on it.
#include <algorithm>
#include <cmath>
#include <vector>

#include "pm_grid.cuh"
#include "pm_launch.h"

using namespace pmd;

namespace {

constexpr int SCAN_BS = 1024;

__global__ void k_keys(const double* __restrict__ pts, int64_t n, double ox, double oy, double oz, double inv_cell, int ncx,
                       int ncy, int ncz, int nbx, int nby, int32_t* __restrict__ key, int32_t* __restrict__ rank,
                       int32_t* __restrict__ count) {
  int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= n) return;
  double p[3] = {pts[3 * i], pts[3 * i + 1], pts[3 * i + 2]};
  double o[3] = {ox, oy, oz};
  int nc[3] = {ncx, ncy, ncz};
  int c[3];
  for (int a = 0; a < 3; a++) {
    double f = floor((p[a] - o[a]) * inv_cell);
    c[a] = !(f >= 0) ? 0 : (f > nc[a] - 1 ? nc[a] - 1 : (int)f);  // NaN -> 0
  }
  int b = (c[0] / PM_GRID_B) + nbx * ((c[1] / PM_GRID_B) + nby * (c[2] / PM_GRID_B));
  int l = (c[0] % PM_GRID_B) + PM_GRID_B * ((c[1] % PM_GRID_B) + PM_GRID_B * (c[2] % PM_GRID_B));
  int k = b * PM_GRID_CELLS_PER_BLOCK + l;
  key[i] = k;
  rank[i] = atomicAdd(count + k, 1);
}

// exclusive scan, phase 1: per-block scan + block sums
__global__ void k_scan_local(const int32_t* __restrict__ in, int64_t n, int32_t* __restrict__ out, int32_t* __restrict__ sums) {
  __shared__ int32_t buf[SCAN_BS];
  int64_t i = blockIdx.x * (int64_t)SCAN_BS + threadIdx.x;
  int32_t v = i < n ? in[i] : 0;
  buf[threadIdx.x] = v;
  __syncthreads();
  for (int off = 1; off < SCAN_BS; off <<= 1) {
    int32_t t = threadIdx.x >= off ? buf[threadIdx.x - off] : 0;
    __syncthreads();
    buf[threadIdx.x] += t;
    __syncthreads();
  }
  if (i < n) out[i] = buf[threadIdx.x] - v;
  if (threadIdx.x == SCAN_BS - 1) sums[blockIdx.x] = buf[threadIdx.x];
}
__global__ void k_scan_add(int32_t* __restrict__ out, int64_t n, const int32_t* __restrict__ offs) {
  int64_t i = blockIdx.x * (int64_t)SCAN_BS + threadIdx.x;
  if (i < n) out[i] += offs[blockIdx.x];
}

// exclusive scan of n int32 into out (out may alias nothing); uses tmp allocations
cudaError_t exclusive_scan(const int32_t* in, int64_t n, int32_t* out, cudaStream_t s, std::vector<void*>& tmp) {
  int64_t nb = (n + SCAN_BS - 1) / SCAN_BS;
  int32_t* sums = nullptr;
  cudaError_t e = cudaMalloc(&sums, (size_t)(nb + 1) * sizeof(int32_t));
  if (e != cudaSuccess) return e;
  tmp.push_back(sums);
  k_scan_local<<<(unsigned)nb, SCAN_BS, 0, s>>>(in, n, out, sums);
  if ((e = cudaGetLastError()) != cudaSuccess) return e;
  if (nb > 1) {
    int32_t* offs = nullptr;
    if ((e = cudaMalloc(&offs, (size_t)(nb + 1) * sizeof(int32_t))) != cudaSuccess) return e;
    tmp.push_back(offs);
    if ((e = exclusive_scan(sums, nb, offs, s, tmp)) != cudaSuccess) return e;
    k_scan_add<<<(unsigned)nb, SCAN_BS, 0, s>>>(out, n, offs);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
  }
  return cudaSuccess;
}

__global__ void k_scatter(const double* __restrict__ pts, int64_t n, const int32_t* __restrict__ key, const int32_t* __restrict__ rank,
                          const int32_t* __restrict__ start, double* __restrict__ px, double* __restrict__ py, double* __restrict__ pz,
                          float4* __restrict__ p32) {
  int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= n) return;
  int pos = start[key[i]] + rank[i];
  double x = pts[3 * i], y = pts[3 * i + 1], z = pts[3 * i + 2];
  px[pos] = x;
  py[pos] = y;
  pz[pos] = z;
  p32[pos] = make_float4((float)x, (float)y, (float)z, 0.0f);
}

__global__ void k_flags(const int32_t* __restrict__ count, int64_t nc, int32_t* __restrict__ flag) {
  int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i < nc) flag[i] = count[i] > 0 ? 1 : 0;
}

__global__ void k_cell_records(const int32_t* __restrict__ count, const int32_t* __restrict__ start, const int32_t* __restrict__ recidx,
                               int64_t nc, const double* __restrict__ px, const double* __restrict__ py, const double* __restrict__ pz,
                               float* __restrict__ cell_box, int32_t* __restrict__ cell_pts, float4* __restrict__ cell_rec) {
  int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (c >= nc || count[c] == 0) return;
  int r = recidx[c];
  int p0 = start[c], p1 = p0 + count[c];
  double lo[3] = {INFINITY, INFINITY, INFINITY}, hi[3] = {-INFINITY, -INFINITY, -INFINITY};
  for (int i = p0; i < p1; i++) {
    double v[3] = {px[i], py[i], pz[i]};
    for (int a = 0; a < 3; a++) {
      lo[a] = fmin(lo[a], v[a]);
      hi[a] = fmax(hi[a], v[a]);
    }
  }
  for (int a = 0; a < 3; a++) {
    cell_box[6 * r + a] = __double2float_rd(lo[a]);
    cell_box[6 * r + 3 + a] = __double2float_ru(hi[a]);
  }
  cell_pts[2 * r] = p0;
  cell_pts[2 * r + 1] = p1;
  cell_rec[2 * r] = make_float4(cell_box[6 * r], cell_box[6 * r + 1], cell_box[6 * r + 2], __int_as_float(p0));
  cell_rec[2 * r + 1] = make_float4(cell_box[6 * r + 3], cell_box[6 * r + 4], cell_box[6 * r + 5], __int_as_float(p1));
}

__global__ void k_block_records(const int32_t* __restrict__ recidx_ex, int64_t nblocks, int32_t n_rec, const float* __restrict__ cell_box,
                                int32_t* __restrict__ blk_occ, float* __restrict__ blk_box) {
  int64_t b = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (b >= nblocks) return;
  int r0 = recidx_ex[b * PM_GRID_CELLS_PER_BLOCK];
  int r1 = (b + 1 < nblocks) ? recidx_ex[(b + 1) * PM_GRID_CELLS_PER_BLOCK] : n_rec;
  blk_occ[2 * b] = r0;
  blk_occ[2 * b + 1] = r1;
  float lo[3] = {INFINITY, INFINITY, INFINITY}, hi[3] = {-INFINITY, -INFINITY, -INFINITY};
  for (int r = r0; r < r1; r++)
    for (int a = 0; a < 3; a++) {
      lo[a] = fminf(lo[a], cell_box[6 * r + a]);
      hi[a] = fmaxf(hi[a], cell_box[6 * r + 3 + a]);
    }
  for (int a = 0; a < 3; a++) {
    blk_box[6 * b + a] = lo[a];
    blk_box[6 * b + 3 + a] = hi[a];
  }
}

// Chebyshev (L-infinity) distance transform of the block occupancy, separable: one pass per
// axis, each line scanned in O(n^2) (n <= a few hundred blocks).
__global__ void k_edf_pass(const int32_t* __restrict__ blk_occ, const int16_t* __restrict__ in, int16_t* __restrict__ out, int nbx, int nby,
                           int nbz, int axis) {
  const int n[3] = {nbx, nby, nbz};
  const int a1 = axis == 0 ? 1 : 0, a2 = axis == 2 ? 1 : 2;
  int line = blockIdx.x * blockDim.x + threadIdx.x;
  if (line >= n[a1] * n[a2]) return;
  int c[3];
  c[a1] = line % n[a1];
  c[a2] = line / n[a1];
  const int len = n[axis];
  for (int i = 0; i < len; i++) {
    int best = 32767;
    for (int j = 0; j < len; j++) {
      c[axis] = j;
      const int b = c[0] + nbx * (c[1] + nby * c[2]);
      int v;
      if (axis == 0) {
        v = blk_occ[2 * b] < blk_occ[2 * b + 1] ? 0 : 32767;
      } else {
        v = in[b];
      }
      if (v == 32767) continue;
      const int d = max(abs(i - j), v);
      best = min(best, d);
    }
    c[axis] = i;
    out[c[0] + nbx * (c[1] + nby * c[2])] = (int16_t)best;
  }
}
// occupancy of fine cells in x-fastest order (counts are stored block-major)
__global__ void k_cell_occ(const int32_t* __restrict__ count, int ncx, int ncy, int ncz, int nbx, int nby, uint8_t* __restrict__ occ) {
  int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= (int64_t)ncx * ncy * ncz) return;
  const int cx = (int)(i % ncx), cy = (int)((i / ncx) % ncy), cz = (int)(i / ((int64_t)ncx * ncy));
  const int b = (cx / PM_GRID_B) + nbx * ((cy / PM_GRID_B) + nby * (cz / PM_GRID_B));
  const int l = (cx % PM_GRID_B) + PM_GRID_B * ((cy % PM_GRID_B) + PM_GRID_B * (cz % PM_GRID_B));
  occ[i] = count[(int64_t)b * PM_GRID_CELLS_PER_BLOCK + l] > 0 ? 1 : 0;
}
// Separable squared distance transform between cell boxes: per-axis cost max(|i - j| - 1, 0)^2
// summed over axes (the squared gap between two unit cells), minimised over occupied cells.
__global__ void k_bdt_pass(const uint8_t* __restrict__ occ, const int32_t* __restrict__ in, int32_t* __restrict__ out, int nx, int ny,
                           int nz, int axis) {
  const int n[3] = {nx, ny, nz};
  const int a1 = axis == 0 ? 1 : 0, a2 = axis == 2 ? 1 : 2;
  int line = blockIdx.x * blockDim.x + threadIdx.x;
  if (line >= n[a1] * n[a2]) return;
  int c[3];
  c[a1] = line % n[a1];
  c[a2] = line / n[a1];
  c[axis] = 0;
  const int len = n[axis];
  const int64_t stride = axis == 0 ? 1 : (axis == 1 ? (int64_t)nx : (int64_t)nx * ny);
  const int64_t base = c[0] + (int64_t)nx * (c[1] + (int64_t)ny * c[2]);
  const int INF = 0x3fffffff;
  for (int i = 0; i < len; i++) {
    int best = INF;
    for (int j = 0; j < len; j++) {
      const int64_t b = base + j * stride;
      const int v = axis == 0 ? (occ[b] ? 0 : INF) : in[b];
      if (v >= INF) continue;
      const int gap = max(abs(i - j) - 1, 0);
      best = min(best, v + gap * gap);
    }
    out[base + i * stride] = best;
  }
}
__global__ void k_bdt_final(const int32_t* __restrict__ d2, int64_t n, double cell, float* __restrict__ lb) {
  int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= n) return;
  lb[i] = d2[i] >= 0x3fffffff ? INFINITY : __double2float_rd(sqrt((double)d2[i]) * cell);
}
__global__ void k_edf_final(const int16_t* __restrict__ in, int64_t n, uint8_t* __restrict__ edf) {
  int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i < n) edf[i] = (uint8_t)min((int)in[i], 255);
}

// Nearest-point field: per fine cell, the exact FP32 nearest point of the cell centre within
// `reach` and a lower bound on the centre's distance to every point (the FP32 value shrunk by the
// rounding of d^2, of the square root and of the FP32 point coordinates).  Cells whose
// box-to-box bound already reaches `reach` skip the search.
__global__ void k_field(PmGridDev G, int ncx, int ncy, int ncz, float reach, int2* __restrict__ out, float4* __restrict__ out_np,
                        uint16_t* __restrict__ out16) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= (int64_t)ncx * ncy * ncz) return;
  const int cx = (int)(i % ncx), cy = (int)((i / ncx) % ncy), cz = (int)(i / ((int64_t)ncx * ncy));
  const float x = field_centre(G.o32[0], cx, G.cell32), y = field_centre(G.o32[1], cy, G.cell32),
              z = field_centre(G.o32[2], cz, G.cell32);
  const float slack = 4e-6f + 2e-7f * (fabsf(x) + fabsf(y) + fabsf(z));
  float d = reach;
  int idx = -1;
  if (G.cell_lb[i] < reach) {
    const NNResult32 r = grid_nearest32(G, x, y, z, reach * reach);
    if (r.idx >= 0) {
      d = sqrtf(r.d2);
      idx = r.idx;
    }
  }
  const float lb = fmaxf(d * (1.0f - 1e-6f) - slack, 0.0f);
  out[i] = make_int2(__float_as_int(lb), idx);
  // the same bound in 16 bits, rounded down to PM_FIELD16_UNIT (capped: the cap is a lower bound too)
  const float u = floorf(lb * (1.0f / PM_FIELD16_UNIT) * (1.0f - 1e-6f));
  out16[i] = (uint16_t)(u >= 65535.f ? 65535.f : (u > 0.f ? u : 0.f));
  float4 np = make_float4(0.f, 0.f, 0.f, __int_as_float(-1));
  if (idx >= 0) {
    np = G.p32[idx];
    np.w = __int_as_float(idx);
  }
  out_np[i] = np;
}

// Per-block candidate lists.  For a block whose cells all have a nearest point in the field, a
// query q inside it (up to FP32 rounding of its block) has a point within
//   ub(q) = |q - p(c)| <= |q - c| + |c - p(c)| <= half cell diagonal + d(c)
// for its field cell c (inside the block or a neighbour, taken over the block's cells plus a one-cell
// shell), so the exact search needs only the occupied blocks within R_B = max(d(c)) + 1.5 cell
// diagonals of the block's box.  Pass 0: R_B and the list length; pass 1 (after a scan): the
// lists, sorted by box distance.
__device__ __forceinline__ float box_box_d(const float* a_lo, const float* a_hi, const float* b) {
  float d2 = 0.f;
  for (int k = 0; k < 3; k++) {
    const float g = fmaxf(fmaxf(b[k] - a_hi[k], a_lo[k] - b[3 + k]), 0.f);
    d2 = fmaf(g, g, d2);
  }
  return sqrtf(d2);
}
__global__ void k_blk_lists(PmGridDev G, int pass, float reach_cap, float* __restrict__ R, int32_t* __restrict__ cnt,
                            const int32_t* __restrict__ start, int2* __restrict__ cand) {
  const int nbx = G.nbx, nby = G.nby, nbz = G.nbz;
  const int64_t b = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (b >= (int64_t)nbx * nby * nbz) return;
  const int bx = (int)(b % nbx), by = (int)((b / nbx) % nby), bz = (int)(b / ((int64_t)nbx * nby));
  const float cell = G.cell32;
  float rb;
  if (pass == 0) {
    const int nc[3] = {nbx * PM_GRID_B, nby * PM_GRID_B, nbz * PM_GRID_B};
    float dmax = 0.f;
    bool ok = true;
    for (int cz = bz * PM_GRID_B - 1; cz <= (bz + 1) * PM_GRID_B && ok; cz++)
      for (int cy = by * PM_GRID_B - 1; cy <= (by + 1) * PM_GRID_B && ok; cy++)
        for (int cx = bx * PM_GRID_B - 1; cx <= (bx + 1) * PM_GRID_B; cx++) {
          if (cx < 0 || cy < 0 || cz < 0 || cx >= nc[0] || cy >= nc[1] || cz >= nc[2]) continue;
          const int2 nn = G.cell_nn[cx + (int64_t)nc[0] * (cy + (int64_t)nc[1] * cz)];
          if (nn.y < 0) {
            ok = false;
            break;
          }
          // |c - p(c)| with the FP32 expression of the queries' upper bound
          const float4 p = G.p32[nn.y];
          const float dx = p.x - field_centre(G.o32[0], cx, cell), dy = p.y - field_centre(G.o32[1], cy, cell),
                      dz = p.z - field_centre(G.o32[2], cz, cell);
          dmax = fmaxf(dmax, sqrtf(fmaf(dx, dx, fmaf(dy, dy, dz * dz))));
        }
    rb = ok ? dmax * 1.00001f + 1.5f * 1.7320508f * cell + 1e-5f : -1.f;
    if (!(rb <= reach_cap)) rb = -1.f;  // far from the cloud: no list, the walk handles it
    R[b] = rb;
  } else {
    rb = R[b];
  }
  if (rb < 0.f) {
    if (pass == 0) cnt[b] = 0;
    return;
  }
  const float blk = G.blk32;
  const float slack = 1e-5f;
  const float lo[3] = {G.o32[0] + (float)bx * blk - slack, G.o32[1] + (float)by * blk - slack, G.o32[2] + (float)bz * blk - slack};
  const float hi[3] = {lo[0] + blk + 2.f * slack, lo[1] + blk + 2.f * slack, lo[2] + blk + 2.f * slack};
  const int k = (int)ceilf(rb / blk) + 1;
  int n = 0;
  const int32_t s0 = pass == 1 ? start[b] : 0;
  for (int z = max(bz - k, 0); z <= min(bz + k, nbz - 1); z++)
    for (int y = max(by - k, 0); y <= min(by + k, nby - 1); y++)
      for (int x = max(bx - k, 0); x <= min(bx + k, nbx - 1); x++) {
        const int64_t o = x + (int64_t)nbx * (y + (int64_t)nby * z);
        const int2 occ = reinterpret_cast<const int2*>(G.blk_occ)[o];
        if (occ.x >= occ.y) continue;
        const float d = box_box_d(lo, hi, G.blk_box + 6 * o);
        if (!(d < rb * 1.00001f + 1e-6f)) continue;
        if (pass == 1) {  // insertion by distance
          int j = n;
          while (j > 0) {
            if (__int_as_float(cand[s0 + j - 1].y) <= d) break;
            cand[s0 + j] = cand[s0 + j - 1];
            j--;
          }
          cand[s0 + j] = make_int2((int32_t)o, __float_as_int(d));
        }
        n++;
      }
  if (pass == 0) cnt[b] = n;
}

// The candidate lists widened for the warp searches: each entry also carries its block's
// occupied-cell range and box, read with the entry instead of one dependent load later.
__global__ void k_cand_expand(const int2* __restrict__ cand, int64_t n, const int32_t* __restrict__ blk_occ,
                              const float* __restrict__ blk_box, int4* __restrict__ cand4, float4* __restrict__ cand_box) {
  const int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (k >= n) return;
  const int2 e = cand[k];
  const int b = e.x;
  cand4[k] = make_int4(blk_occ[2 * b], blk_occ[2 * b + 1], b, e.y);
  const float* x = blk_box + 6 * (int64_t)b;
  cand_box[2 * k] = make_float4(x[0], x[1], x[2], 0.f);
  cand_box[2 * k + 1] = make_float4(x[3], x[4], x[5], 0.f);
}

__global__ void k_blk_ranges(const float* __restrict__ R, const int32_t* __restrict__ cnt, const int32_t* __restrict__ start, int64_t nb,
                             int2* __restrict__ out) {
  const int64_t b = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (b >= nb) return;
  out[b] = R[b] < 0.f ? make_int2(-1, -1) : make_int2(start[b], start[b] + cnt[b]);
}

// Per-fine-cell lists of occupied cells, built per grid block (one CTA of kClThreads, 64 fine
// cells).  A query q in cell c (up to the FP32 rounding of its cell, covered by 1e-5 m of slack on
// the cell's box) has a point within
//   ub(c) = |q - p(c)| <= half cell diagonal + |c - p(c)|
// (p(c): the nearest point of the cell centre, from the field), so only the occupied cells whose
// box lies within ub(c) of c's box can hold its nearest point.  The CTA stages in shared memory
// the occupied cells within U = max ub(c) of the block's box, found on the block's candidate list
// (which covers blk_reach >= U); each warp then takes fine cells of the block and filters the
// staged cells by their distance from the cell's box.  Cells without a field point, with ub(c)
// above list_reach or beyond their block's reach, and the cells of a block whose candidates do
// not fit kClStage get no list (the queries there take the block walk).
// pass 0: count per cell (0: no list) and the 64-bit total; pass 1: the entries, unsorted into
// tmp, then ranked by (distance, record) into out.
constexpr int kClThreads = 256;
constexpr int kClStage = 3072;  // staged candidate cells per block (28 B each)
constexpr size_t kClSmem = (size_t)kClStage * 28;
__global__ void __launch_bounds__(kClThreads) k_cell_lists(PmGridDev G, int pass, float list_reach, int32_t* __restrict__ cnt,
                                                           const int32_t* __restrict__ start, uint2* __restrict__ tmp,
                                                           uint32_t* __restrict__ out, unsigned long long* __restrict__ total) {
  extern __shared__ __align__(16) float cl_smem[];  // kClSmem bytes: the staged boxes, then their records
  float* s_box = cl_smem;
  int* s_id = reinterpret_cast<int*>(cl_smem + kClStage * 6);
  __shared__ float s_ub[PM_GRID_CELLS_PER_BLOCK];
  __shared__ int s_n, s_umax, s_over;
  const unsigned FULL = 0xffffffffu;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int64_t b = blockIdx.x;
  const int bx = (int)(b % G.nbx), by = (int)((b / G.nbx) % G.nby), bz = (int)(b / ((int64_t)G.nbx * G.nby));
  const int nc[3] = {G.nbx * PM_GRID_B, G.nby * PM_GRID_B, G.nbz * PM_GRID_B};
  const float cell = G.cell32;
  const int2 rng = G.blk_list[b];
  const float rb = G.blk_reach[b];
  if (tid == 0) {
    s_n = 0;
    s_umax = 0;
    s_over = 0;
  }
  __syncthreads();
  // 1. ub per fine cell of the block (local index x fastest), -1: no list
  auto cell_index = [&](int l, int& cx, int& cy, int& cz) {
    cx = bx * PM_GRID_B + l % PM_GRID_B;
    cy = by * PM_GRID_B + (l / PM_GRID_B) % PM_GRID_B;
    cz = bz * PM_GRID_B + l / (PM_GRID_B * PM_GRID_B);
    return cx + (int64_t)nc[0] * (cy + (int64_t)nc[1] * cz);
  };
  if (tid < PM_GRID_CELLS_PER_BLOCK) {
    int cx, cy, cz;
    const int64_t i = cell_index(tid, cx, cy, cz);
    const int2 nn = G.cell_nn[i];
    float ub = -1.f;
    if (nn.y >= 0 && rng.x >= 0) {
      const float4 p = G.p32[nn.y];
      const float dx = p.x - field_centre(G.o32[0], cx, cell), dy = p.y - field_centre(G.o32[1], cy, cell),
                  dz = p.z - field_centre(G.o32[2], cz, cell);
      ub = sqrtf(fmaf(dx, dx, fmaf(dy, dy, dz * dz))) * 1.00001f + 0.8660254f * cell * 1.00001f + 3e-5f;
      if (!(ub <= list_reach) || !(ub <= rb)) ub = -1.f;
    }
    s_ub[tid] = ub;
    if (ub >= 0.f) atomicMax(&s_umax, __float_as_int(ub));  // non-negative floats order as their bits
  }
  __syncthreads();
  const float U = __int_as_float(s_umax);
  if (U <= 0.f) {  // block-uniform: no cell of the block gets a list
    if (pass == 0 && tid < PM_GRID_CELLS_PER_BLOCK) {
      int cx, cy, cz;
      cnt[cell_index(tid, cx, cy, cz)] = 0;
    }
    return;
  }
  // 2. stage the occupied cells within U of the block's box (entries sorted by block distance)
  const float slack = 1e-5f, blk = G.blk32;
  const float blo[3] = {G.o32[0] + (float)bx * blk - slack, G.o32[1] + (float)by * blk - slack, G.o32[2] + (float)bz * blk - slack};
  const float bhi[3] = {blo[0] + blk + 2.f * slack, blo[1] + blk + 2.f * slack, blo[2] + blk + 2.f * slack};
  for (int k = rng.x + warp; k < rng.y; k += kClThreads / 32) {  // warp per entry
    const int4 e = G.cand4[k];
    if (__int_as_float(e.w) > U * 1.0001f + 1e-6f) break;  // warp-uniform; later entries are farther
    for (int base = e.x; base < e.y; base += 32) {
      const int o = base + lane;
      if (o < e.y) {
        const float* cb = G.cell_box + 6 * (int64_t)o;
        if (box_box_d(blo, bhi, cb) * (1.0f - 1e-6f) <= U) {
          const int slot = atomicAdd(&s_n, 1);
          if (slot < kClStage) {
            s_id[slot] = o;
            for (int a = 0; a < 6; a++) s_box[6 * slot + a] = cb[a];
          } else {
            s_over = 1;
          }
        }
      }
    }
  }
  __syncthreads();
  const int n_stage = min(s_n, kClStage);
  const bool over = s_over != 0;
  const float to_units = (float)PM_CL_UNITS / cell;
  // 3. per fine cell (warp-strided): filter the staged cells by the distance from the cell's box
  for (int l = warp; l < PM_GRID_CELLS_PER_BLOCK; l += kClThreads / 32) {
    int cx, cy, cz;
    const int64_t i = cell_index(l, cx, cy, cz);
    const float ub = over ? -1.f : s_ub[l];
    if (ub < 0.f) {  // warp-uniform
      if (pass == 0 && lane == 0) cnt[i] = 0;
      continue;
    }
    const int room = pass == 1 ? cnt[i] : 0;  // pass 1 fills the room pass 0 counted
    if (pass == 1 && room <= 0) continue;
    const float lo[3] = {G.o32[0] + (float)cx * cell - slack, G.o32[1] + (float)cy * cell - slack, G.o32[2] + (float)cz * cell - slack};
    const float hi[3] = {lo[0] + cell + 2.f * slack, lo[1] + cell + 2.f * slack, lo[2] + cell + 2.f * slack};
    const int64_t s0 = pass == 1 ? start[i] : 0;
    int n = 0;
    for (int base = 0; base < n_stage; base += 32) {
      const int j = base + lane;
      float d = 0.f;
      bool in = false;
      if (j < n_stage) {
        d = box_box_d(lo, hi, s_box + 6 * j) * (1.0f - 1e-6f);
        in = d <= ub;
      }
      const unsigned bal = __ballot_sync(FULL, in);
      if (pass == 1 && in) {
        const int pos = n + __popc(bal & ((1u << lane) - 1u));
        if (pos < room) tmp[s0 + pos] = make_uint2((unsigned)s_id[j], __float_as_uint(d));
      }
      n += __popc(bal);
    }
    if (pass == 0) {
      if (n > 1024) n = 0;  // a list this long is not worth its scan (or its build-time sort): the cell takes the block walk
      if (lane == 0) {
        cnt[i] = n;
        atomicAdd(total, (unsigned long long)n);  // 64-bit: the int32 scan is used only below 2^30
      }
      continue;
    }
    __syncwarp();
    n = min(n, room);  // equal: both passes stage and filter the same cells
    // rank of each entry by (distance, record): every order has a unique place
    for (int j = lane; j < n; j += 32) {
      const uint2 ej = tmp[s0 + j];
      const float dj = __uint_as_float(ej.y);
      int r = 0;
      for (int k = 0; k < n; k++) {
        const uint2 ek = tmp[s0 + k];
        const float dk = __uint_as_float(ek.y);
        r += (dk < dj || (dk == dj && ek.x < ej.x)) ? 1 : 0;
      }
      const float u = floorf(dj * to_units * (1.0f - 1e-6f));
      const unsigned q = u >= 255.f ? 255u : (u > 0.f ? (unsigned)u : 0u);
      out[s0 + r] = ej.x | (q << 24);
    }
    // should the passes ever differ, the rest of the room still holds valid records (record 0 at the
    // largest bound)
    for (int j = n + lane; j < room; j += 32) out[s0 + j] = 0u | (255u << 24);
    __syncwarp();
  }
}

__global__ void k_cl_ranges(const int32_t* __restrict__ cnt, const int32_t* __restrict__ start, int64_t n, int2* __restrict__ out) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= n) return;
  out[i] = cnt[i] > 0 ? make_int2(start[i], start[i] + cnt[i]) : make_int2(-1, -1);
}

inline unsigned nblk(int64_t n, int bs) { return (unsigned)((n + bs - 1) / bs); }
// FP32 roundings of a double toward -inf / +inf (host)
inline float round_down_f(double v) {
  float f = (float)v;
  if ((double)f > v) f = std::nextafter(f, -INFINITY);
  return f;
}
inline float round_up_f(double v) {
  float f = (float)v;
  if ((double)f < v) f = std::nextafter(f, INFINITY);
  return f;
}

}  // namespace

namespace pmg {

void grid_free(GridBuild& g) {
  for (int i = 0; i < g.n_allocs; i++) cudaFree(g.allocs[i]);
  g.n_allocs = 0;
}

cudaError_t grid_build(GridBuild& g, cudaStream_t s) {
  std::vector<void*> tmp;
  cudaError_t e = cudaSuccess;
  g.n_allocs = 0;
  g.bytes = 0;
  auto keep = [&](size_t bytes, void** p) -> cudaError_t {
    if (g.n_allocs >= (int)(sizeof(g.allocs) / sizeof(g.allocs[0]))) return cudaErrorMemoryAllocation;
    cudaError_t r = cudaMalloc(p, bytes < 16 ? 16 : bytes);
    if (r == cudaSuccess) {
      g.allocs[g.n_allocs++] = *p;
      g.bytes += (int64_t)(bytes < 16 ? 16 : bytes);
    }
    return r;
  };
  auto scratch = [&](size_t bytes, void** p) -> cudaError_t {
    cudaError_t r = cudaMalloc(p, bytes < 16 ? 16 : bytes);
    if (r == cudaSuccess) tmp.push_back(*p);
    return r;
  };
  PmGridDev& d = g.dev;
  const int64_t n = g.n;
  // the caller sizes the grid (origin, blocks per axis, block edge); refuse a descriptor whose
  // cell keys would fall outside the count arrays
  if (!(d.nbx >= 1 && d.nby >= 1 && d.nbz >= 1 && n >= 0 && g.cell > 0.0 && d.block > 0.0 && g.field_reach > 0.0) ||
      (int64_t)d.nbx * d.nby * d.nbz * PM_GRID_CELLS_PER_BLOCK > ((int64_t)1 << 30))
    return cudaErrorInvalidValue;
  for (int a = 0; a < 3; a++) {
    d.o32[a] = (float)d.origin[a];
    d.box_lo32[a] = round_down_f(d.lb[a] + d.radius);
    d.box_hi32[a] = round_up_f(d.ub[a] - d.radius);
  }
  d.blk32 = (float)d.block;
  d.inv_blk32 = (float)(1.0 / d.block);
  d.cell32 = (float)(d.block / PM_GRID_B);
  d.inv_cell32 = (float)(PM_GRID_B / d.block);
  const int nb[3] = {d.nbx, d.nby, d.nbz};
  const int nc[3] = {nb[0] * PM_GRID_B, nb[1] * PM_GRID_B, nb[2] * PM_GRID_B};
  const int64_t nblocks = (int64_t)nb[0] * nb[1] * nb[2];
  const int64_t ncells = nblocks * PM_GRID_CELLS_PER_BLOCK;
  int32_t *key = nullptr, *rank = nullptr, *count = nullptr, *start = nullptr, *flag = nullptr, *recidx = nullptr;
  double *px = nullptr, *py = nullptr, *pz = nullptr;
  float4* p32 = nullptr;
  int32_t *blk_occ = nullptr, *cell_pts = nullptr;
  uint8_t* edf = nullptr;
  float* cell_lb = nullptr;
  int2* cell_nn = nullptr;
  uint16_t* cell_lb16 = nullptr;
  float4* cell_np = nullptr;
  float4* cell_rec = nullptr;
  int4* cand4 = nullptr;
  float4* cand_box = nullptr;
  int2* blk_list = nullptr;
  int2* blk_cand = nullptr;
  int2* cl_rng = nullptr;
  uint32_t* cl_ent = nullptr;
  int64_t n_cl = 0;
  int2* sb_rng = nullptr;
  int32_t* sb_blk = nullptr;
  float* sb_box = nullptr;
  int32_t n_sb = 0;
  float* blk_reach = nullptr;
  int32_t n_cand = 0;
  float *blk_box = nullptr, *cell_box = nullptr;
  int32_t n_rec = 0;
  do {
    if ((e = scratch(n * 4, (void**)&key)) != cudaSuccess) break;
    if ((e = scratch(n * 4, (void**)&rank)) != cudaSuccess) break;
    if ((e = scratch(ncells * 4, (void**)&count)) != cudaSuccess) break;
    if ((e = scratch(ncells * 4, (void**)&start)) != cudaSuccess) break;
    if ((e = scratch(ncells * 4, (void**)&flag)) != cudaSuccess) break;
    if ((e = scratch(ncells * 4, (void**)&recidx)) != cudaSuccess) break;
    if ((e = keep(n * 8, (void**)&px)) != cudaSuccess) break;
    if ((e = keep(n * 8, (void**)&py)) != cudaSuccess) break;
    if ((e = keep(n * 8, (void**)&pz)) != cudaSuccess) break;
    if ((e = keep(n * 16, (void**)&p32)) != cudaSuccess) break;
    if ((e = keep(nblocks * 8, (void**)&blk_occ)) != cudaSuccess) break;
    if ((e = keep(nblocks * 24, (void**)&blk_box)) != cudaSuccess) break;
    if ((e = cudaMemsetAsync(count, 0, ncells * 4, s)) != cudaSuccess) break;
    if (n > 0) {
      k_keys<<<nblk(n, 256), 256, 0, s>>>(g.pts, n, d.origin[0], d.origin[1], d.origin[2], 1.0 / g.cell, nc[0], nc[1], nc[2], nb[0],
                                           nb[1], key, rank, count);
      if ((e = cudaGetLastError()) != cudaSuccess) break;
    }
    if ((e = exclusive_scan(count, ncells, start, s, tmp)) != cudaSuccess) break;
    if (n > 0) {
      k_scatter<<<nblk(n, 256), 256, 0, s>>>(g.pts, n, key, rank, start, px, py, pz, p32);
      if ((e = cudaGetLastError()) != cudaSuccess) break;
    }
    k_flags<<<nblk(ncells, 256), 256, 0, s>>>(count, ncells, flag);
    if ((e = cudaGetLastError()) != cudaSuccess) break;
    if ((e = exclusive_scan(flag, ncells, recidx, s, tmp)) != cudaSuccess) break;
    int32_t last_idx = 0, last_flag = 0;
    if ((e = cudaMemcpyAsync(&last_idx, recidx + ncells - 1, 4, cudaMemcpyDeviceToHost, s)) != cudaSuccess) break;
    if ((e = cudaMemcpyAsync(&last_flag, flag + ncells - 1, 4, cudaMemcpyDeviceToHost, s)) != cudaSuccess) break;
    if ((e = cudaStreamSynchronize(s)) != cudaSuccess) break;
    n_rec = last_idx + last_flag;
    if ((e = keep((size_t)n_rec * 24, (void**)&cell_box)) != cudaSuccess) break;
    if ((e = keep((size_t)n_rec * 8, (void**)&cell_pts)) != cudaSuccess) break;
    if ((e = keep((size_t)std::max<int32_t>(n_rec, 1) * 32, (void**)&cell_rec)) != cudaSuccess) break;
    k_cell_records<<<nblk(ncells, 256), 256, 0, s>>>(count, start, recidx, ncells, px, py, pz, cell_box, cell_pts, cell_rec);
    if ((e = cudaGetLastError()) != cudaSuccess) break;
    k_block_records<<<nblk(nblocks, 128), 128, 0, s>>>(recidx, nblocks, n_rec, cell_box, blk_occ, blk_box);
    if ((e = cudaGetLastError()) != cudaSuccess) break;
    {  // super-blocks of PM_GRID_SB^3 blocks (host: a few thousand at most): the non-empty ones, each
       // with its occupied blocks and the box of its points
      std::vector<int32_t> h_occ((size_t)nblocks * 2);
      std::vector<float> h_box((size_t)nblocks * 6);
      if ((e = cudaMemcpyAsync(h_occ.data(), blk_occ, h_occ.size() * 4, cudaMemcpyDeviceToHost, s)) != cudaSuccess) break;
      if ((e = cudaMemcpyAsync(h_box.data(), blk_box, h_box.size() * 4, cudaMemcpyDeviceToHost, s)) != cudaSuccess) break;
      if ((e = cudaStreamSynchronize(s)) != cudaSuccess) break;
      const int ns[3] = {(nb[0] + PM_GRID_SB - 1) / PM_GRID_SB, (nb[1] + PM_GRID_SB - 1) / PM_GRID_SB, (nb[2] + PM_GRID_SB - 1) / PM_GRID_SB};
      std::vector<std::vector<int32_t>> members((size_t)ns[0] * ns[1] * ns[2]);
      for (int64_t b = 0; b < nblocks; b++) {
        if (h_occ[2 * b] >= h_occ[2 * b + 1]) continue;
        const int bx = (int)(b % nb[0]), by = (int)((b / nb[0]) % nb[1]), bz = (int)(b / ((int64_t)nb[0] * nb[1]));
        members[(bx / PM_GRID_SB) + (size_t)ns[0] * ((by / PM_GRID_SB) + (size_t)ns[1] * (bz / PM_GRID_SB))].push_back((int32_t)b);
      }
      std::vector<int2> h_rng;
      std::vector<int32_t> h_blk;
      std::vector<float> h_sbox;
      for (auto& m : members) {
        if (m.empty()) continue;
        float lo[3] = {INFINITY, INFINITY, INFINITY}, hi[3] = {-INFINITY, -INFINITY, -INFINITY};
        for (int32_t b : m)
          for (int a = 0; a < 3; a++) {
            lo[a] = std::min(lo[a], h_box[6 * (size_t)b + a]);
            hi[a] = std::max(hi[a], h_box[6 * (size_t)b + 3 + a]);
          }
        h_rng.push_back(make_int2((int)h_blk.size(), (int)(h_blk.size() + m.size())));
        h_blk.insert(h_blk.end(), m.begin(), m.end());
        for (int a = 0; a < 3; a++) h_sbox.push_back(lo[a]);
        for (int a = 0; a < 3; a++) h_sbox.push_back(hi[a]);
      }
      n_sb = (int32_t)h_rng.size();
      if ((e = keep(std::max<size_t>(h_rng.size(), 1) * 8, (void**)&sb_rng)) != cudaSuccess) break;
      if ((e = keep(std::max<size_t>(h_blk.size(), 1) * 4, (void**)&sb_blk)) != cudaSuccess) break;
      if ((e = keep(std::max<size_t>(h_sbox.size(), 1) * 4, (void**)&sb_box)) != cudaSuccess) break;
      if (n_sb > 0) {
        if ((e = cudaMemcpyAsync(sb_rng, h_rng.data(), h_rng.size() * 8, cudaMemcpyHostToDevice, s)) != cudaSuccess) break;
        if ((e = cudaMemcpyAsync(sb_blk, h_blk.data(), h_blk.size() * 4, cudaMemcpyHostToDevice, s)) != cudaSuccess) break;
        if ((e = cudaMemcpyAsync(sb_box, h_sbox.data(), h_sbox.size() * 4, cudaMemcpyHostToDevice, s)) != cudaSuccess) break;
        if ((e = cudaStreamSynchronize(s)) != cudaSuccess) break;  // the host vectors go out of scope
      }
    }
    {
      int16_t *t0 = nullptr, *t1 = nullptr;
      if ((e = scratch(nblocks * 2, (void**)&t0)) != cudaSuccess) break;
      if ((e = scratch(nblocks * 2, (void**)&t1)) != cudaSuccess) break;
      if ((e = keep(nblocks, (void**)&edf)) != cudaSuccess) break;
      k_edf_pass<<<nblk((int64_t)nb[1] * nb[2], 64), 64, 0, s>>>(blk_occ, nullptr, t0, nb[0], nb[1], nb[2], 0);
      k_edf_pass<<<nblk((int64_t)nb[0] * nb[2], 64), 64, 0, s>>>(blk_occ, t0, t1, nb[0], nb[1], nb[2], 1);
      k_edf_pass<<<nblk((int64_t)nb[0] * nb[1], 64), 64, 0, s>>>(blk_occ, t1, t0, nb[0], nb[1], nb[2], 2);
      k_edf_final<<<nblk(nblocks, 256), 256, 0, s>>>(t0, nblocks, edf);
      if ((e = cudaGetLastError()) != cudaSuccess) break;
    }
    {  // Euclidean lower-bound field on fine cells
      const int64_t ncl = (int64_t)nc[0] * nc[1] * nc[2];
      int32_t *t0 = nullptr, *t1 = nullptr;
      uint8_t* occ = nullptr;
      if ((e = scratch(ncl * 4, (void**)&t0)) != cudaSuccess) break;
      if ((e = scratch(ncl * 4, (void**)&t1)) != cudaSuccess) break;
      if ((e = scratch(ncl, (void**)&occ)) != cudaSuccess) break;
      if ((e = keep(ncl * 4, (void**)&cell_lb)) != cudaSuccess) break;
      k_cell_occ<<<nblk(ncl, 256), 256, 0, s>>>(count, nc[0], nc[1], nc[2], nb[0], nb[1], occ);
      k_bdt_pass<<<nblk((int64_t)nc[1] * nc[2], 64), 64, 0, s>>>(occ, nullptr, t0, nc[0], nc[1], nc[2], 0);
      k_bdt_pass<<<nblk((int64_t)nc[0] * nc[2], 64), 64, 0, s>>>(occ, t0, t1, nc[0], nc[1], nc[2], 1);
      k_bdt_pass<<<nblk((int64_t)nc[0] * nc[1], 64), 64, 0, s>>>(occ, t1, t0, nc[0], nc[1], nc[2], 2);
      k_bdt_final<<<nblk(ncl, 256), 256, 0, s>>>(t0, ncl, g.cell, cell_lb);
      if ((e = cudaGetLastError()) != cudaSuccess) break;
    }
    {  // nearest-point field (needs the finished descriptor for its nearest-neighbour walks)
      const int64_t ncl = (int64_t)nc[0] * nc[1] * nc[2];
      if ((e = keep(ncl * 8, (void**)&cell_nn)) != cudaSuccess) break;
      if ((e = keep(ncl * 2, (void**)&cell_lb16)) != cudaSuccess) break;
      if ((e = keep(ncl * 16, (void**)&cell_np)) != cudaSuccess) break;
      PmGridDev v = d;
      v.blk_list = nullptr;  // the walks below run without candidate lists
      v.blk_cand = nullptr;
      v.blk_reach = nullptr;
      v.cand4 = nullptr;
      v.cand_box = nullptr;
      v.cl_rng = nullptr;
      v.cl_ent = nullptr;
      v.sb_rng = sb_rng;
      v.sb_blk = sb_blk;
      v.sb_box = sb_box;
      v.n_sb = n_sb;
      v.px = px;
      v.py = py;
      v.pz = pz;
      v.p32 = p32;
      v.blk_occ = blk_occ;
      v.blk_box = blk_box;
      v.cell_box = cell_box;
      v.cell_pts = cell_pts;
      v.cell_rec = cell_rec;
      v.edf = edf;
      v.cell_lb = cell_lb;
      v.n_points = (int32_t)n;
      k_field<<<nblk(ncl, 128), 128, 0, s>>>(v, nc[0], nc[1], nc[2], (float)g.field_reach, cell_nn, cell_np, cell_lb16);
      if ((e = cudaGetLastError()) != cudaSuccess) break;
      // per-block candidate lists
      v.cell_nn = cell_nn;
      v.cell_np = cell_np;
      v.cell_lb16 = cell_lb16;
      int32_t *cnt = nullptr, *lstart = nullptr;
      if ((e = keep(nblocks * 4, (void**)&blk_reach)) != cudaSuccess) break;
      if ((e = keep(nblocks * 8, (void**)&blk_list)) != cudaSuccess) break;
      if ((e = scratch(nblocks * 4, (void**)&cnt)) != cudaSuccess) break;
      if ((e = scratch(nblocks * 4, (void**)&lstart)) != cudaSuccess) break;
      k_blk_lists<<<nblk(nblocks, 128), 128, 0, s>>>(v, 0, (float)g.field_reach, blk_reach, cnt, nullptr, nullptr);
      if ((e = cudaGetLastError()) != cudaSuccess) break;
      if ((e = exclusive_scan(cnt, nblocks, lstart, s, tmp)) != cudaSuccess) break;
      int32_t last_start = 0, last_cnt = 0;
      if ((e = cudaMemcpyAsync(&last_start, lstart + nblocks - 1, 4, cudaMemcpyDeviceToHost, s)) != cudaSuccess) break;
      if ((e = cudaMemcpyAsync(&last_cnt, cnt + nblocks - 1, 4, cudaMemcpyDeviceToHost, s)) != cudaSuccess) break;
      if ((e = cudaStreamSynchronize(s)) != cudaSuccess) break;
      n_cand = last_start + last_cnt;
      if ((e = keep((size_t)std::max<int32_t>(n_cand, 1) * 8, (void**)&blk_cand)) != cudaSuccess) break;
      k_blk_lists<<<nblk(nblocks, 128), 128, 0, s>>>(v, 1, (float)g.field_reach, blk_reach, cnt, lstart, blk_cand);
      k_blk_ranges<<<nblk(nblocks, 256), 256, 0, s>>>(blk_reach, cnt, lstart, nblocks, blk_list);
      if ((e = keep((size_t)std::max<int32_t>(n_cand, 1) * 16, (void**)&cand4)) != cudaSuccess) break;
      if ((e = keep((size_t)std::max<int32_t>(n_cand, 1) * 32, (void**)&cand_box)) != cudaSuccess) break;
      if (n_cand > 0) k_cand_expand<<<nblk(n_cand, 256), 256, 0, s>>>(blk_cand, n_cand, blk_occ, blk_box, cand4, cand_box);
      if ((e = cudaGetLastError()) != cudaSuccess) break;
      // per-fine-cell lists (record indices must fit their 24 bits); ncl: the fine cells, as above
      if ((e = keep((size_t)ncl * 8, (void**)&cl_rng)) != cudaSuccess) break;
      if (g.list_reach > 0.0 && n_rec < (1 << 24) && n_cand > 0) {
        v.blk_list = blk_list;
        v.blk_cand = blk_cand;
        v.blk_reach = blk_reach;
        v.cand4 = cand4;
        v.cand_box = cand_box;
        int32_t *ccnt = nullptr, *cstart = nullptr;
        unsigned long long* ctot = nullptr;
        if ((e = scratch((size_t)ncl * 4, (void**)&ccnt)) != cudaSuccess) break;
        if ((e = scratch((size_t)ncl * 4, (void**)&cstart)) != cudaSuccess) break;
        if ((e = scratch(8, (void**)&ctot)) != cudaSuccess) break;
        if ((e = cudaMemsetAsync(ctot, 0, 8, s)) != cudaSuccess) break;
        if ((e = cudaFuncSetAttribute(k_cell_lists, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kClSmem)) != cudaSuccess) break;
        k_cell_lists<<<(unsigned)nblocks, kClThreads, kClSmem, s>>>(v, 0, (float)g.list_reach, ccnt, nullptr, nullptr, nullptr, ctot);
        if ((e = cudaGetLastError()) != cudaSuccess) break;
        unsigned long long total = 0;
        if ((e = cudaMemcpyAsync(&total, ctot, 8, cudaMemcpyDeviceToHost, s)) != cudaSuccess) break;
        if ((e = cudaStreamSynchronize(s)) != cudaSuccess) break;
        n_cl = (int64_t)total;
        uint2* cl_tmp = nullptr;
        if (n_cl > 0 && n_cl < ((int64_t)1 << 30)) {  // the int32 scan below holds it
          if ((e = exclusive_scan(ccnt, ncl, cstart, s, tmp)) != cudaSuccess) break;
          if ((e = keep((size_t)n_cl * 4, (void**)&cl_ent)) != cudaSuccess) break;
          if ((e = scratch((size_t)n_cl * 8, (void**)&cl_tmp)) != cudaSuccess) break;
          k_cell_lists<<<(unsigned)nblocks, kClThreads, kClSmem, s>>>(v, 1, (float)g.list_reach, ccnt, cstart, cl_tmp, cl_ent, nullptr);
          if ((e = cudaGetLastError()) != cudaSuccess) break;
          k_cl_ranges<<<nblk(ncl, 256), 256, 0, s>>>(ccnt, cstart, ncl, cl_rng);
        } else {
          n_cl = 0;
          if ((e = cudaMemsetAsync(cl_rng, 0xff, (size_t)ncl * 8, s)) != cudaSuccess) break;
        }
      } else {
        if ((e = cudaMemsetAsync(cl_rng, 0xff, (size_t)ncl * 8, s)) != cudaSuccess) break;
      }
      if ((e = cudaGetLastError()) != cudaSuccess) break;
    }
    e = cudaStreamSynchronize(s);
  } while (false);
  for (void* p : tmp) cudaFree(p);
  if (e != cudaSuccess) {
    grid_free(g);
    return e;
  }
  d.px = px;
  d.py = py;
  d.pz = pz;
  d.p32 = p32;
  d.blk_occ = blk_occ;
  d.blk_box = blk_box;
  d.cell_box = cell_box;
  d.cell_pts = cell_pts;
  d.cell_rec = cell_rec;
  d.edf = edf;
  d.cell_lb = cell_lb;
  d.cell_nn = cell_nn;
  d.cell_np = cell_np;
  d.cell_lb16 = cell_lb16;
  d.blk_list = blk_list;
  d.blk_cand = blk_cand;
  d.blk_reach = blk_reach;
  d.cand4 = cand4;
  d.cand_box = cand_box;
  d.cl_rng = cl_rng;
  d.cl_ent = cl_ent;
  d.sb_rng = sb_rng;
  d.sb_blk = sb_blk;
  d.sb_box = sb_box;
  d.n_sb = n_sb;
  g.n_cell_list = n_cl;
  g.n_occupied = n_rec;
  g.n_cand = n_cand;
  d.field_reach = (float)g.field_reach;
  d.n_points = (int32_t)n;
  return cudaSuccess;
}

}  // namespace pmg
