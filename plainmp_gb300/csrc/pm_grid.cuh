// Exact nearest-neighbour queries on the device point-cloud grid (replaces the KD-tree of
// collision/kdtree.cpp:67-96 inside CloudSDF::evaluate, primitive_sdf.hpp:597-599).
//
// Layout (built by k_grid.cu): blocks of PM_GRID_B^3 fine cells; each occupied fine cell has
// a conservative FP32 bounding box of its points (lo rounded down, hi rounded up) and a
// contiguous point range; each block has the union box and its range of occupied-cell
// records; super-blocks of PM_GRID_SB^3 blocks list their occupied blocks.  Near the cloud,
// a fine cell's list names every occupied cell that can hold the nearest point of a query
// inside it, nearest first, and a query scans it until the stored lower bound reaches the best
// distance.  Elsewhere the FP64 query visits the super-blocks by box distance, and the bounded
// FP32 query walks Chebyshev rings of blocks around the query's (clamped) block; both skip
// boxes at least as far as the best distance so far.
//
// Exactness: the squared distance of a point is fl(dx*dx + (dy*dy + dz*dz)) with d = p - q,
// as the KD-tree computes it (kdtree.cpp:125).  The box distance uses the same formula on
// per-axis gaps that are never larger than the gap to any point in the box, and rounding is
// monotone, so a pruned box holds no point with a smaller squared distance: the returned
// value is exactly min_i fl(|p_i - q|^2), the KD-tree's value.  Among exactly equidistant
// points the nearest point returned may differ from the KD-tree's.
#pragma once
#include "pm_common.h"
#include "pm_math.cuh"


namespace pmd {

__device__ __forceinline__ double gap64(double q, double lo, double hi) {
  if (q < lo) return lo - q;
  if (q > hi) return q - hi;
  return 0.0;
}
__device__ __forceinline__ double box_d2_64(const float* b, const D3& q) {
  double gx = gap64(q.x, (double)b[0], (double)b[3]);
  double gy = gap64(q.y, (double)b[1], (double)b[4]);
  double gz = gap64(q.z, (double)b[2], (double)b[5]);
  return gx * gx + (gy * gy + gz * gz);
}

struct NNResult64 {
  double d2;
  int32_t idx;  // sorted point index, -1 if the cloud is empty
};

// The fine cell of q (FP32 arithmetic, the expression the cell lists were built against) and its
// cell list range; false where q lies outside the grid or its cell has no list.
__device__ __forceinline__ bool cell_list_of(const PmGridDev& G, float qx, float qy, float qz, int2& rng) {
  if (G.cl_rng == nullptr) return false;
  const float qa[3] = {qx, qy, qz};
  const int nc[3] = {G.nbx * PM_GRID_B, G.nby * PM_GRID_B, G.nbz * PM_GRID_B};
  int cc[3];
  for (int a = 0; a < 3; a++) {
    const float t = floorf((qa[a] - G.o32[a]) * G.inv_cell32);
    if (!(t >= 0.f && t <= (float)(nc[a] - 1))) return false;
    cc[a] = (int)t;
  }
  rng = __ldg(G.cl_rng + (cc[0] + nc[0] * (cc[1] + (int64_t)nc[1] * cc[2])));
  return rng.x >= 0;
}

// FP64 scan of q's cell list (nearest first; the scan ends at the first entry whose stored lower
// bound reaches the best).  The list holds every occupied cell that can contain q's nearest point
// (built with 3e-5 m of slack, far above the FP32 / FP64 difference of q's cell assignment), so
// the result is the global exact minimum.
__device__ inline bool list_nearest64(const PmGridDev& G, const D3& q, NNResult64& r) {
  int2 rng;
  if (!cell_list_of(G, (float)q.x, (float)q.y, (float)q.z, rng)) return false;
  const double unit = (double)G.cell32 * (1.0 / PM_CL_UNITS);
  for (int k = rng.x; k < rng.y; k++) {
    const uint32_t e = __ldg(G.cl_ent + k);
    const double lbd = (double)(e >> 24) * unit;
    if (lbd * lbd * (1.0 - 1e-9) >= r.d2) break;  // sorted: no later entry comes closer
    const int c = (int)(e & 0xffffffu);
    if (box_d2_64(G.cell_box + 6 * (int64_t)c, q) >= r.d2) continue;
    const int p0 = G.cell_pts[2 * c], p1 = G.cell_pts[2 * c + 1];
    for (int i = p0; i < p1; i++) {
      D3 d{G.px[i] - q.x, G.py[i] - q.y, G.pz[i] - q.z};
      double d2 = d.x * d.x + (d.y * d.y + d.z * d.z);
      if (d2 < r.d2) {
        r.d2 = d2;
        r.idx = i;
      }
    }
  }
  return true;
}

// FP64 search over the super-blocks, for queries without a cell list (far from the cloud or
// outside the grid): the super-block with the smallest box distance first, then every other
// super-block whose box is closer than the best; inside one, its occupied blocks, their cells and
// points, each skipped when its box is not closer than the best.
__device__ inline void sb_nearest64(const PmGridDev& G, const D3& q, NNResult64& r) {
  auto visit = [&](int j) {
    const int2 br = __ldg(G.sb_rng + j);
    for (int k = br.x; k < br.y; k++) {
      const int b = __ldg(G.sb_blk + k);
      if (box_d2_64(G.blk_box + 6 * (int64_t)b, q) >= r.d2) continue;
      const int c0 = G.blk_occ[2 * b], c1 = G.blk_occ[2 * b + 1];
      for (int c = c0; c < c1; c++) {
        if (box_d2_64(G.cell_box + 6 * (int64_t)c, q) >= r.d2) continue;
        const int p0 = G.cell_pts[2 * c], p1 = G.cell_pts[2 * c + 1];
        for (int i = p0; i < p1; i++) {
          D3 d{G.px[i] - q.x, G.py[i] - q.y, G.pz[i] - q.z};
          double d2 = d.x * d.x + (d.y * d.y + d.z * d.z);
          if (d2 < r.d2) {
            r.d2 = d2;
            r.idx = i;
          }
        }
      }
    }
  };
  double lb_min = INFINITY;
  int j_min = -1;
  for (int j = 0; j < G.n_sb; j++) {
    const double lb = box_d2_64(G.sb_box + 6 * (int64_t)j, q);
    if (lb < lb_min) {
      lb_min = lb;
      j_min = j;
    }
  }
  if (j_min < 0 || !(lb_min < r.d2)) return;
  visit(j_min);
  for (int j = 0; j < G.n_sb; j++)
    if (j != j_min && box_d2_64(G.sb_box + 6 * (int64_t)j, q) < r.d2) visit(j);
}

// Exact FP64 nearest squared distance among the points with squared distance below maxd2
// (idx = -1 when there is none): q's cell list where it has one, else the super-blocks.
__device__ inline NNResult64 grid_nearest64(const PmGridDev& G, const D3& q, double maxd2 = INFINITY) {
  NNResult64 r{maxd2, -1};
  // a NaN or infinite query is farther than every bound from every point (the KD-tree's
  // comparisons all fail the same way); it must not reach the index arithmetic below
  if (G.n_points <= 0 || !isfinite(q.x) || !isfinite(q.y) || !isfinite(q.z)) return r;
  if (list_nearest64(G, q, r)) return r;
  sb_nearest64(G, q, r);
  return r;
}

// FP32 variant: same walk in single precision.  Returns the exact minimum over points of the
// FP32-evaluated squared distance (same monotonicity argument).
struct NNResult32 {
  float d2;
  int32_t idx;
};
__device__ __forceinline__ float gap32(float q, float lo, float hi) { return fmaxf(fmaxf(lo - q, q - hi), 0.0f); }
__device__ __forceinline__ float box_d2_32(const float* b, float qx, float qy, float qz) {
  float gx = gap32(qx, b[0], b[3]), gy = gap32(qy, b[1], b[4]), gz = gap32(qz, b[2], b[5]);
  return fmaf(gx, gx, fmaf(gy, gy, gz * gz));
}
// maxd2 bounds the search: points at squared distance >= maxd2 are never reported (idx stays -1
// when none is closer).
__device__ inline NNResult32 grid_nearest32(const PmGridDev& G, float qx, float qy, float qz, float maxd2 = INFINITY) {
  NNResult32 r{maxd2, -1};
  if (G.n_points <= 0 || !isfinite(qx) || !isfinite(qy) || !isfinite(qz)) return r;  // as grid_nearest64
  int2 crng;
  if (cell_list_of(G, qx, qy, qz, crng)) {  // q's cell list: every cell that can hold its nearest point
    const float unit = G.cell32 * (1.0f / (float)PM_CL_UNITS);
    for (int k = crng.x; k < crng.y; k++) {
      const uint32_t e = __ldg(G.cl_ent + k);
      const float lbd = (float)(e >> 24) * unit;
      if (lbd * lbd * (1.0f - 1e-5f) >= r.d2) break;
      const int c = (int)(e & 0xffffffu);
      const float4 lo = __ldg(G.cell_rec + 2 * c), hi = __ldg(G.cell_rec + 2 * c + 1);
      const float gx = gap32(qx, lo.x, hi.x), gy = gap32(qy, lo.y, hi.y), gz = gap32(qz, lo.z, hi.z);
      if (fmaf(gx, gx, fmaf(gy, gy, gz * gz)) >= r.d2) continue;
      for (int i = __float_as_int(lo.w); i < __float_as_int(hi.w); i++) {
        const float4 p = __ldg(G.p32 + i);
        const float dx = p.x - qx, dy = p.y - qy, dz = p.z - qz;
        const float d2 = fmaf(dx, dx, fmaf(dy, dy, dz * dz));
        if (d2 < r.d2 || (d2 == r.d2 && r.idx >= 0 && i < r.idx)) {
          r.d2 = d2;
          r.idx = i;
        }
      }
    }
    return r;
  }
  const float inv = G.inv_blk32;
  const float ox = G.o32[0], oy = G.o32[1], oz = G.o32[2];
  const float blk = G.blk32;
  const float qa[3] = {qx, qy, qz};
  const float oa[3] = {ox, oy, oz};
  const int nb[3] = {G.nbx, G.nby, G.nbz};
  int cb[3];
  bool inside = true;
  for (int a = 0; a < 3; a++) {
    float f = floorf((qa[a] - oa[a]) * inv);
    if (!(f >= 0.f && f <= (float)(nb[a] - 1))) inside = false;
    cb[a] = !(f >= 0.f) ? 0 : (f > (float)(nb[a] - 1) ? nb[a] - 1 : (int)f);
  }
  if (inside && G.blk_list) {  // the block's candidate list covers every point within its reach
    const int b = cb[0] + nb[0] * (cb[1] + nb[1] * cb[2]);
    const int2 rng = __ldg(G.blk_list + b);
    if (rng.x >= 0 && sqrtf(r.d2) <= __ldg(G.blk_reach + b)) {
      for (int k = rng.x; k < rng.y; k++) {
        const int2 e = __ldg(G.blk_cand + k);
        const float ed = __int_as_float(e.y);
        if (ed * ed * (1.0f - 1e-5f) >= r.d2) break;  // sorted: no later entry can be closer
        const int bb = e.x;
        if (box_d2_32(G.blk_box + 6 * bb, qx, qy, qz) >= r.d2) continue;
        const int2 occ = __ldg(reinterpret_cast<const int2*>(G.blk_occ) + bb);
        for (int c = occ.x; c < occ.y; c++) {
          if (box_d2_32(G.cell_box + 6 * c, qx, qy, qz) >= r.d2) continue;
          const int2 pr = __ldg(reinterpret_cast<const int2*>(G.cell_pts) + c);
          for (int i = pr.x; i < pr.y; i++) {
            const float4 p = __ldg(G.p32 + i);
            const float dx = p.x - qx, dy = p.y - qy, dz = p.z - qz;
            const float d2 = fmaf(dx, dx, fmaf(dy, dy, dz * dz));
            if (d2 < r.d2) {
              r.d2 = d2;
              r.idx = i;
            }
          }
        }
      }
      return r;
    }
  }
  const int k0 = __ldg(G.edf + cb[0] + nb[0] * (cb[1] + nb[1] * cb[2]));
  if (inside && k0 >= 2) {
    const float lb0 = (float)(k0 - 1) * blk - 4e-6f;
    if (lb0 > 0.f && lb0 * lb0 >= r.d2) return r;
  }
  const int kmax = max(nb[0], max(nb[1], nb[2]));
  for (int K = min(k0, kmax); K <= kmax; K++) {
    const int z0 = max(cb[2] - K, 0), z1 = min(cb[2] + K, nb[2] - 1);
    const int y0 = max(cb[1] - K, 0), y1 = min(cb[1] + K, nb[1] - 1);
    const int x0 = max(cb[0] - K, 0), x1 = min(cb[0] + K, nb[0] - 1);
    for (int bz = z0; bz <= z1; bz++) {
      const bool zf = (bz == cb[2] - K) || (bz == cb[2] + K);
      for (int by = y0; by <= y1; by++) {
        const bool yf = zf || (by == cb[1] - K) || (by == cb[1] + K);
        const int step = yf ? 1 : 2 * K;
        for (int bx = (yf ? x0 : cb[0] - K); bx <= x1; bx += (step > 0 ? step : 1)) {
          if (bx < x0) continue;
          const int b = bx + nb[0] * (by + nb[1] * bz);
          const int2 occ = __ldg(reinterpret_cast<const int2*>(G.blk_occ) + b);
          if (occ.x >= occ.y) continue;
          if (box_d2_32(G.blk_box + 6 * b, qx, qy, qz) >= r.d2) continue;
          for (int c = occ.x; c < occ.y; c++) {
            if (box_d2_32(G.cell_box + 6 * c, qx, qy, qz) >= r.d2) continue;
            const int2 pr = __ldg(reinterpret_cast<const int2*>(G.cell_pts) + c);
            for (int i = pr.x; i < pr.y; i++) {
              float4 p = __ldg(G.p32 + i);
              float dx = p.x - qx, dy = p.y - qy, dz = p.z - qz;
              float d2 = fmaf(dx, dx, fmaf(dy, dy, dz * dz));
              if (d2 < r.d2) {
                r.d2 = d2;
                r.idx = i;
              }
            }
          }
          if (K == 0) break;
        }
      }
    }
    float lb = INFINITY;
    for (int a = 0; a < 3; a++) {
      if (cb[a] - K - 1 >= 0) lb = fminf(lb, qa[a] - (oa[a] + (float)(cb[a] - K) * blk));
      if (cb[a] + K + 1 <= nb[a] - 1) lb = fminf(lb, (oa[a] + (float)(cb[a] + K + 1) * blk) - qa[a]);
    }
    if (lb == INFINITY) break;
    // face positions carry FP32 rounding (< 1e-6 m inside a few-metre workspace)
    const float lbm = lb - 4e-6f;
    if (lbm > 0.f && lbm * lbm >= r.d2) break;
  }
  return r;
}

// Centre of fine cell c along one axis.  The build and the queries evaluate this same FP32
// expression, so a query measures its offset from exactly the point whose distance was stored.
__device__ __forceinline__ float field_centre(float origin, int c, float cellf) { return origin + ((float)c + 0.5f) * cellf; }

// Nearest-point field of a query q: lb = a lower bound on the distance from q to any point, by the
// triangle inequality from the distance of a fine-cell centre c (lb = d(c) - |q - c|, any cell
// would do; the containing one is the tightest); idx = the nearest point of that centre, an upper
// bound candidate (-1 if none within field_reach, and outside the grid).  Outside the grid, lb is
// the distance to the box of the points.
// With want_np, np = that point's record (x y z, w = index bits), read in parallel with the bound.
struct FieldLB {
  float lb;
  int idx;
  float4 np;
};
__device__ __forceinline__ FieldLB grid_field32(const PmGridDev& G, float qx, float qy, float qz, bool want_np = false) {
  FieldLB f{INFINITY, -1, make_float4(0.f, 0.f, 0.f, 0.f)};
  if (G.n_points <= 0) return f;
  const float cellf = G.cell32;
  const float inv = G.inv_cell32;
  const float qa[3] = {qx, qy, qz};
  const int nc[3] = {G.nbx * PM_GRID_B, G.nby * PM_GRID_B, G.nbz * PM_GRID_B};
  int cc[3];
  bool inside = true;
  for (int a = 0; a < 3; a++) {
    const float t = floorf((qa[a] - G.o32[a]) * inv);
    if (!(t >= 0.f && t <= (float)(nc[a] - 1))) inside = false;
    cc[a] = inside ? (int)t : 0;
  }
  if (!inside) {
    float d2 = 0.f;
    for (int a = 0; a < 3; a++) {
      const float lo = G.box_lo32[a], hi = G.box_hi32[a];
      const float gap = fmaxf(fmaxf(lo - qa[a], qa[a] - hi), 0.f);
      d2 = fmaf(gap, gap, d2);
    }
    f.lb = fmaxf(sqrtf(d2) * (1.0f - 1e-6f) - 4e-6f, 0.f);
    return f;
  }
  const int64_t ci = cc[0] + nc[0] * (cc[1] + (int64_t)nc[1] * cc[2]);
  const int2 nn = __ldg(G.cell_nn + ci);
  if (want_np) f.np = __ldg(G.cell_np + ci);
  const float dx = qx - field_centre(G.o32[0], cc[0], cellf), dy = qy - field_centre(G.o32[1], cc[1], cellf),
              dz = qz - field_centre(G.o32[2], cc[2], cellf);
  const float off = sqrtf(fmaf(dx, dx, fmaf(dy, dy, dz * dz))) * (1.0f + 1e-6f) + 1e-7f;
  f.lb = fmaxf(__int_as_float(nn.x) - off, 0.f);
  f.idx = nn.y;
  return f;
}

// grid_field32's lower bound from the 16-bit copy of the field (at most PM_FIELD16_UNIT looser): one
// 2-byte load, for the checks that need no nearest point.
__device__ __forceinline__ float grid_field_lb16(const PmGridDev& G, float qx, float qy, float qz) {
  if (G.n_points <= 0) return INFINITY;
  const float cellf = G.cell32;
  const float qa[3] = {qx, qy, qz};
  const int nc[3] = {G.nbx * PM_GRID_B, G.nby * PM_GRID_B, G.nbz * PM_GRID_B};
  int cc[3];
  bool inside = true;
  for (int a = 0; a < 3; a++) {
    const float t = floorf((qa[a] - G.o32[a]) * G.inv_cell32);
    if (!(t >= 0.f && t <= (float)(nc[a] - 1))) inside = false;
    cc[a] = inside ? (int)t : 0;
  }
  if (!inside) {  // as grid_field32: the distance to the box of the points
    float d2 = 0.f;
    for (int a = 0; a < 3; a++) {
      const float gap = fmaxf(fmaxf(G.box_lo32[a] - qa[a], qa[a] - G.box_hi32[a]), 0.f);
      d2 = fmaf(gap, gap, d2);
    }
    return fmaxf(sqrtf(d2) * (1.0f - 1e-6f) - 4e-6f, 0.f);
  }
  const unsigned short u = __ldg(G.cell_lb16 + (cc[0] + nc[0] * (cc[1] + (int64_t)nc[1] * cc[2])));
  const float dx = qx - field_centre(G.o32[0], cc[0], cellf), dy = qy - field_centre(G.o32[1], cc[1], cellf),
              dz = qz - field_centre(G.o32[2], cc[2], cellf);
  const float off = sqrtf(fmaf(dx, dx, fmaf(dy, dy, dz * dz))) * (1.0f + 1e-6f) + 1e-7f;
  return fmaxf((float)u * PM_FIELD16_UNIT * (1.0f - 1e-6f) - off, 0.f);
}

// FP32 squared distance from q to point idx, the expression of every nearest-neighbour walk.
__device__ __forceinline__ float point_d2_32(const PmGridDev& G, int idx, float qx, float qy, float qz) {
  const float4 p = __ldg(G.p32 + idx);
  const float dx = p.x - qx, dy = p.y - qy, dz = p.z - qz;
  return fmaf(dx, dx, fmaf(dy, dy, dz * dz));
}

}  // namespace pmd
