// FP32 fast path with FP64 recheck (validity booleans identical to the plain method).
//
// Per block of CPB configurations (k_fast_valid; k_fast_edges over the waypoints of edges):
//   1. FK in FP32 into shared memory, with a running bound on each slot's error against the
//      FP64 FK of the reference (see fk32); every later margin adds the bound of the spheres
//      involved.  A configuration with a non-finite coordinate goes to the exact FP64 check;
//   2. group culling: the clearance of each sphere group's bounding sphere against each
//      primitive (a point cloud: the lower bound of its nearest-point field);
//   3. sphere tasks (sphere x primitive) and self-pair tasks (a group test per lane, then the
//      surviving group pairs by the whole warp), each decision a tri-state of an FP32 clearance g
//      against a margin m derived from the FP32 error bound: pass if g > m, fail if g < -m,
//      otherwise the term is queued.  Spheres near a point cloud need its exact nearest point:
//      a warp-cooperative search over the block's candidate list, in the block, or with
//      distances in k_hard_queries over a global queue;
//   4. k_fast_recheck evaluates every queued term with the exact FP64 gate-and-test of the
//      reference (primitive_sphere_collision.cpp:191-254) and clears the configuration if the
//      term collides; configurations (edges) whose terms did not fit the queue get the full
//      FP64 check.
// Why the terms suffice: ext collision = OR over groups g and primitives p of
// [gate(g,p) AND OR_s test(s,p)] = OR over (s,p) of [gate(g(s),p) AND test(s,p)]; a sphere
// that certainly collides by more than the margin lies inside its group sphere, whose gate then
// also fails, so certain terms need no FP64 work.  Self pairs factor the same way.
#include <algorithm>
#include <cmath>
#include <map>
#include <mutex>
#include <vector>

#include "pm_grad.cuh"
#include "pm_launch.h"
#include "pm_view.cuh"

using namespace pmd;

namespace {

constexpr float kU = 5.9604645e-8f;  // 2^-24
// Margin of an FP32 clearance: 64 units of roundoff of the magnitudes involved, plus 1 um.  The
// error analysis of the FP32 evaluation (pose rounding, one dot product, one square root)
// gives about 52 units for the box, the largest case.
__device__ __forceinline__ float margin32(float mag) { return 1e-6f + 64.0f * kU * (1.0f + mag); }

struct PrimF {
  int kind, aa, za, cloud;
  float lb[3], ub[3], pos[3], rot[9];
  float a, b, c, mag;
};
struct SphereF {
  float x, y, z, r;
  int group, tiny;  // tiny: the FP64 radius is below 1e-6 (the reference's special cases)
  float sn;         // |offset in the link frame|, rounded up (for the FK error bound)
};
struct GroupF {
  float rel[3], radius;
  int slot, begin, count, only_self;
  int tiny;
  float gn;  // |group centre in the link frame|, rounded up
  int pad[2];
};

// FP32 FK slot: the local transform's constant part (joint origin, or the fixed transform of a
// slot without a control joint, taken from the model state when the block starts).
struct SlotF {
  int parent, mode, qcol, lid;
  int split;  // PmSlot::split: the FK phase and thread that compute this slot
  float axis[3];
  float lq[4];
  float lt[3];
  float lt1;  // |lt|_1 (prismatic: of the origin part)
};
// Per slot and configuration in shared memory: [0..8] R, [9..11] t, [12] et = bound on |t - t64|,
// [13] eb = bound on |R - R64| as an operator (8 eq + 24 u), [14..17] world quaternion,
// [18] eq = bound on |q - q64|_2.  A point s of the link frame then lies within et + eb |s| of
// its FP64 position, plus the rounding of R s + t that margin32 covers.
constexpr int kPoseF = 20;

enum { ST_PASS = 0, ST_FAIL = 1, ST_MAYBE = 2 };
constexpr int FLAG_FAIL = 1;

// A hard cloud query handed from k_fast_valid to k_hard_queries (distances mode): the sphere centre
// and search reach, then (configuration, sphere | primitive << 16 | validity check << 31, FK error
// bound of the centre as float bits, 0).
struct HardQuery {
  float4 a;
  int4 b;
};

struct Scratch {
  int4* items;
  unsigned int* count;
  unsigned int cap;
  uint8_t* overflow;
  unsigned long long* stats;
  HardQuery* hq;           // global hard-query queue (distances mode), or null: queries stay in the block
  unsigned long long* hq_count;  // entries reserved (64-bit: a large batch may reserve more than 2^32)
  unsigned int hq_cap;
  int st_log2;             // sphere tile: log2 of the spheres a warp row of sphere tasks holds (0: the
                           // least, 32 / configurations per block)
  PmLinkBounds bnd = PmLinkBounds{nullptr, 0};  // a composite constraint's link-position bounds
};

__device__ __forceinline__ float3 xf(const float* P, float x, float y, float z) {  // R (row-major 9) * v + t (P[9..11])
  return make_float3(fmaf(P[0], x, fmaf(P[1], y, fmaf(P[2], z, P[9]))), fmaf(P[3], x, fmaf(P[4], y, fmaf(P[5], z, P[10]))),
                     fmaf(P[6], x, fmaf(P[7], y, fmaf(P[8], z, P[11]))));
}

// compute_approx_sin_cos (kinematics/algorithm.cpp:50-86) with the range reduction in FP64 and
// the polynomial in FP32 (Horner form): within 8 units of roundoff (sin) and 12 (cos) of the FP64
// value for the reduced |x| <= pi/2.
// isfinite of a double by its exponent bits (integer instructions only)
__device__ __forceinline__ bool finite64(double v) { return (__double2hiint(v) & 0x7ff00000) != 0x7ff00000; }

// qf = (float)q: for |q| below pi no range reduction applies, and x = q / 2 rounds to qf / 2 exactly
// (halving commutes with rounding), so the FP64 arithmetic is skipped there with the same result.
__device__ __forceinline__ void approx_sin_cos32_q(double q, float qf, float& s, float& c);
__device__ __forceinline__ void approx_sin_cos32(double x, float& s, float& c) {
  const double pi = 3.14159265358979323846, half_pi = pi * 0.5;
  double cos_sign = 1.0;
  if (x > half_pi || x < -half_pi) {
    if (x > pi || x < -pi) x = x - 2 * pi * floor(x * (1.0 / (2 * pi)) + 0.5);
    if (x < -half_pi) {
      x = -x - pi;
      cos_sign = -1.0;
    } else if (x > half_pi) {
      x = -x + pi;
      cos_sign = -1.0;
    }
  }
  const float xf = (float)x, xx = xf * xf;
  s = xf * (1.0f - xx * (1.0f / 6.0f - xx * (1.0f / 120.0f - xx * (1.0f / 5040.0f - xx * (1.0f / 362880.0f)))));
  c = 1.0f - xx * (0.5f - xx * (1.0f / 24.0f - xx * (1.0f / 720.0f - xx * (1.0f / 40320.0f))));
  if (cos_sign < 0.0) c = -c;
}
__device__ __forceinline__ void approx_sin_cos32_q(double q, float qf, float& s, float& c) {
  if (fabsf(qf) <= 3.1415925f) {  // < pi: |q / 2| < pi / 2 in FP64 too
    const float xf = qf * 0.5f, xx = xf * xf;
    s = xf * (1.0f - xx * (1.0f / 6.0f - xx * (1.0f / 120.0f - xx * (1.0f / 5040.0f - xx * (1.0f / 362880.0f)))));
    c = 1.0f - xx * (0.5f - xx * (1.0f / 24.0f - xx * (1.0f / 720.0f - xx * (1.0f / 40320.0f))));
    return;
  }
  approx_sin_cos32(q * 0.5, s, c);
}

// FP32 FK of one configuration into P (n_slots x kPoseF) with error bounds against the FP64 FK
// of the reference (update_kintree + get_link_pose; algorithm.cpp:88-210).  Bounds, u = 2^-24,
// norms 2-norms, quaternions within 1e-3 of unit norm:
//   local rotation: joint quaternion from sin/cos (Taylor: 8u / 12u; sincosf: 2 ulp + the
//     rounding of x) and an FP32 axis: 20u; times the FP32 origin quaternion: 32u;
//   composition q = qp (x) lq: |dq| <= 1.001 (|dqp| + |dlq|) + 8.1u (4-term fused sums);
//   rotation of a vector v by an FP32 matrix of qp: |d(Rv)| <= (8 |dqp| + 24u) |v| (the map
//     q -> R(q)v has derivative norm <= 6.4 |v| at |q| <= 1.001; matrix and product rounding);
//   translation t = tp + R lt: |dt| <= |dtp| + (8 |dqp| + 24u)|lt| + 1.01 u (|tp|_1 + |lt|_1).
// The base pose adds the rounding of q's base entries (and of their half angles).
// Field f of slot i is P[(i * kPoseF + f) * stride] (stride 1: a block's shared memory, one
// configuration's slots in a row).
// list: the slots to compute, in order (one phase of one thread of the two-thread FK), or null: all
// nsl.  The two threads of a configuration walk their own lists in step, so a warp computes both
// threads' k-th slots with one instruction stream.
__device__ __forceinline__ void fk32(const SlotF* __restrict__ S, int nsl, const float* __restrict__ base8, int base_type, int n_ctrl,
                                     const double* __restrict__ q, bool taylor, float* __restrict__ P, int64_t stride = 1,
                                     const unsigned char* list = nullptr) {
  for (int k = 0; k < nsl; k++) {
    const int i = list ? list[k] : k;
    const SlotF s = S[i];
    float* o = P + (int64_t)i * kPoseF * stride;
    FQ wq;
    float wt[3], eq, et;
    if (s.parent < 0) {
      if (base_type == PM_BASE_PLANAR) {
        const double hy = q[n_ctrl + 2] * 0.5;
        float sy, cy;
        sincosf((float)hy, &sy, &cy);
        wq = FQ{0.f, 0.f, sy, cy};
        wt[0] = (float)q[n_ctrl];
        wt[1] = (float)q[n_ctrl + 1];
        wt[2] = 0.f;
        eq = kU * (8.0f + 2.0f * fabsf((float)hy));
      } else if (base_type == PM_BASE_FLOATING) {
        const double hr = q[n_ctrl + 3] * 0.5, hp = q[n_ctrl + 4] * 0.5, hy = q[n_ctrl + 5] * 0.5;
        float sr, cr, sp, cp, sy, cy;
        sincosf((float)hr, &sr, &cr);
        sincosf((float)hp, &sp, &cp);
        sincosf((float)hy, &sy, &cy);
        wq = FQ{sr * cp * cy - cr * sp * sy, cr * sp * cy + sr * cp * sy, cr * cp * sy - sr * sp * cy, cr * cp * cy + sr * sp * sy};
        for (int k = 0; k < 3; k++) wt[k] = (float)q[n_ctrl + k];
        eq = kU * (40.0f + 4.0f * (fabsf((float)hr) + fabsf((float)hp) + fabsf((float)hy)));
      } else {
        wq = FQ{base8[0], base8[1], base8[2], base8[3]};
        for (int k = 0; k < 3; k++) wt[k] = base8[4 + k];
        eq = 2.0f * kU;
      }
      et = kU * (fabsf(wt[0]) + fabsf(wt[1]) + fabsf(wt[2]));
    } else {
      const float* pp = P + (int64_t)s.parent * kPoseF * stride;
      const FQ pq{pp[(14) * stride], pp[(15) * stride], pp[(16) * stride], pp[(17) * stride]};
      FQ lq{0.f, 0.f, 0.f, 1.f};
      float lt[3] = {s.lt[0], s.lt[1], s.lt[2]};
      float el = 0.f, elt = kU * s.lt1, lt1 = s.lt1;
      bool lid = s.lid != 0;
      if (s.mode == PM_FK_STATE) {
        lq = FQ{s.lq[0], s.lq[1], s.lq[2], s.lq[3]};
        el = 2.0f * kU;
      } else if (s.mode == PM_FK_PRIS) {
        const float th = (float)q[s.qcol];
        for (int k = 0; k < 3; k++) lt[k] = fmaf(s.axis[k], th, s.lt[k]);
        lt1 = fabsf(lt[0]) + fabsf(lt[1]) + fabsf(lt[2]);
        elt = 4.0f * kU * (s.lt1 + fabsf(th) * (fabsf(s.axis[0]) + fabsf(s.axis[1]) + fabsf(s.axis[2])));
        lid = true;
      } else {
        const double qd = q[s.qcol];
        const float qf = (float)qd, xf = qf * 0.5f;  // (float)(qd / 2), exactly
        float sn, cs;
        if (taylor) {
          approx_sin_cos32_q(qd, qf, sn, cs);
        } else {
          sincosf(xf, &sn, &cs);
        }
        const FQ jq{sn * s.axis[0], sn * s.axis[1], sn * s.axis[2], cs};
        lq = lid ? jq : fqmul(FQ{s.lq[0], s.lq[1], s.lq[2], s.lq[3]}, jq);
        el = (lid ? 20.0f : 32.0f) * kU + (taylor ? 0.0f : 2.0f * kU * fabsf(xf));
        lid = false;
      }
      wq = lid ? pq : fqmul(pq, lq);
      for (int k = 0; k < 3; k++)
        wt[k] = pp[(9 + k) * stride] + fmaf(pp[(3 * k) * stride], lt[0], fmaf(pp[(3 * k + 1) * stride], lt[1], pp[(3 * k + 2) * stride] * lt[2]));
      const float peq = pp[(18) * stride];
      eq = lid ? peq + el : 1.001f * (peq + el) + 8.1f * kU;
      const float nlt = sqrtf(fmaf(lt[0], lt[0], fmaf(lt[1], lt[1], lt[2] * lt[2]))) * 1.001f;
      et = pp[(12) * stride] + nlt * pp[(13) * stride] + 1.01f * kU * (fabsf(pp[(9) * stride]) + fabsf(pp[(10) * stride]) + fabsf(pp[(11) * stride]) + lt1) + elt;
    }
    float R[9];
    fqmat(wq, R);
    for (int k = 0; k < 9; k++) o[k * stride] = R[k];
    o[9 * stride] = wt[0];
    o[10 * stride] = wt[1];
    o[11 * stride] = wt[2];
    o[12 * stride] = et;
    o[13 * stride] = 8.0f * eq + 24.0f * kU;
    o[14 * stride] = wq.x;
    o[15 * stride] = wq.y;
    o[16 * stride] = wq.z;
    o[17 * stride] = wq.w;
    o[18 * stride] = eq;
  }
}

// Clearance g (the reference reports a collision iff g <= 0, up to its own rounding), the
// evaluate()-based signed distance sd (minus r) and the magnitude for the margin.
__device__ __forceinline__ void clearance(const PrimF& P, const PmGridDev* clouds, float cx, float cy, float cz, float r, bool tiny,
                                          float extra, float& g, float& sd, float& mag) {
  const float dx = cx - P.pos[0], dy = cy - P.pos[1], dz = cz - P.pos[2];
  mag = fabsf(cx) + fabsf(cy) + fabsf(cz) + P.mag;
  switch (P.kind) {
    case PM_SDF_BOX: {
      float lx, ly, lz;
      if (P.aa) {
        lx = dx;
        ly = dy;
        lz = dz;
      } else {
        lx = fmaf(dx, P.rot[0], fmaf(dy, P.rot[3], dz * P.rot[6]));
        ly = fmaf(dx, P.rot[1], fmaf(dy, P.rot[4], dz * P.rot[7]));
        lz = fmaf(dx, P.rot[2], fmaf(dy, P.rot[5], dz * P.rot[8]));
      }
      const float sx = fabsf(lx) - P.a, sy = fabsf(ly) - P.b, sz = fabsf(lz) - P.c;
      const float mx = fmaxf(sx, 0.f), my = fmaxf(sy, 0.f), mz = fmaxf(sz, 0.f);
      const float ext = sqrtf(fmaf(mx, mx, fmaf(my, my, mz * mz)));
      const float ms = fmaxf(sx, fmaxf(sy, sz));
      g = tiny ? ms - r : ext - r;
      sd = ext + fminf(ms, 0.f) - r;
      return;
    }
    case PM_SDF_CYLINDER: {
      float lx, ly, lz;
      if (P.za) {
        lx = dx;
        ly = dy;
        lz = dz;
      } else {
        lx = fmaf(dx, P.rot[0], fmaf(dy, P.rot[3], dz * P.rot[6]));
        ly = fmaf(dx, P.rot[1], fmaf(dy, P.rot[4], dz * P.rot[7]));
        lz = fmaf(dx, P.rot[2], fmaf(dy, P.rot[5], dz * P.rot[8]));
      }
      const float zs = fabsf(lz) - P.c;
      const float rs = sqrtf(fmaf(lx, lx, ly * ly)) - P.a;
      const float a = fmaxf(rs, 0.f), b = fmaxf(zs, 0.f);
      const float ext = sqrtf(fmaf(a, a, b * b));
      g = tiny ? fmaxf(zs - r, rs) : ext - r;
      sd = ext + fminf(fmaxf(rs, zs), 0.f) - r;
      return;
    }
    case PM_SDF_SPHERE: {
      const float d = sqrtf(fmaf(dx, dx, fmaf(dy, dy, dz * dz))) - P.a;
      g = tiny ? d : d - r;
      sd = d - r;
      return;
    }
    case PM_SDF_GROUND: {  // the reference's AABB (z in [0, 0]) is part of its decision
      g = fmaxf(fabsf(cz) - r, cz + P.a - r);
      sd = cz + P.a - r;
      return;
    }
    case PM_SDF_CLOUD: {
      const float reach = P.a + r + extra;
      NNResult32 nn = grid_nearest32(clouds[P.cloud], cx, cy, cz, reach * reach);
      if (nn.idx < 0) {
        g = reach - P.a - r;  // nothing closer than reach
        sd = 3.0e38f;
        mag = fabsf(cx) + fabsf(cy) + fabsf(cz);
        return;
      }
      const float d = sqrtf(nn.d2);
      g = d - P.a - r;
      sd = g;
      mag = fabsf(cx) + fabsf(cy) + fabsf(cz) + d;
      return;
    }
  }
  g = 3.0e38f;
  sd = 3.0e38f;
}

__device__ __forceinline__ unsigned long long nn_key(float d2, int idx) {
  return ((unsigned long long)__float_as_uint(d2) << 32) | (unsigned)idx;
}

// Block offsets (dx, dy, dz) with max |d| <= kOffR, sorted by the minimum distance between two
// blocks at that offset, sqrt(sum max(|d|-1, 0)^2) block edges (c_off_lb).
constexpr int kOffR = 6;
constexpr int kOffN = (2 * kOffR + 1) * (2 * kOffR + 1) * (2 * kOffR + 1);
__device__ char4 c_off[kOffN];     // global memory: lanes read different entries
__device__ float c_off_lb[kOffN];

// The cell-list search of warp_nearest32 (all 32 lanes, the same query): q's fine cell lists every
// occupied cell that can hold q's nearest point, nearest first.  32 entries at a time: an entry
// whose stored lower bound reaches the best so far ends the scan (the list is sorted); the others
// are tested by their box, and the points of the cells that survive are spread over the lanes (a
// warp scan of their counts).  best / bidx: the bound and candidate on entry, the result on return.
// Returns false, touching nothing, where q's cell has no list.  pre: q's list range read ahead
// (field_corner_record), or x = -2 to read it here.
__device__ __forceinline__ bool warp_nearest_list32(const PmGridDev& G, float qx, float qy, float qz, float& best, int& bidx,
                                                    int2 pre = make_int2(-2, -2)) {
  const unsigned FULL = 0xffffffffu;
  const int lane = threadIdx.x & 31;
  int2 rng = pre;
  if (pre.x == -2 && !cell_list_of(G, qx, qy, qz, rng)) return false;
  if (rng.x < 0) return false;
  const float unit = G.cell32 * (1.0f / (float)PM_CL_UNITS);
  for (int base = rng.x; base < rng.y; base += 32) {  // warp-uniform
    const int k = base + lane;
    bool beyond = true;  // this entry, and (sorted) every later one, lies beyond the best
    int2 pr = make_int2(0, 0);
    if (k < rng.y) {
      const uint32_t e = __ldg(G.cl_ent + k);
      const float lbd = (float)(e >> 24) * unit;
      beyond = lbd * lbd * (1.0f - 1e-5f) >= best;
      if (!beyond) {
        const int o = (int)(e & 0xffffffu);
        const float4 lo = __ldg(G.cell_rec + 2 * o), hi = __ldg(G.cell_rec + 2 * o + 1);
        const float gx = gap32(qx, lo.x, hi.x), gy = gap32(qy, lo.y, hi.y), gz = gap32(qz, lo.z, hi.z);
        if (fmaf(gx, gx, fmaf(gy, gy, gz * gz)) < best) pr = make_int2(__float_as_int(lo.w), __float_as_int(hi.w));
      }
    }
    const bool stop = __shfl_sync(FULL, beyond ? 1 : 0, 31) != 0;
    const int n = pr.y - pr.x;
    int incl = n;
    for (int o = 1; o < 32; o <<= 1) {
      const int t = __shfl_up_sync(FULL, incl, o);
      if (lane >= o) incl += t;
    }
    const int total = __shfl_sync(FULL, incl, 31);
    for (int t0 = 0; t0 < total; t0 += 32) {  // warp-uniform
      const int t = t0 + lane;
      int lo = 0, hi = 31;  // owner: the first lane whose inclusive count exceeds t
      for (int it = 0; it < 5; it++) {
        const int mid = (lo + hi) >> 1;
        if (__shfl_sync(FULL, incl, mid) <= t) lo = mid + 1;
        else hi = mid;
      }
      const int own_first = __shfl_sync(FULL, pr.x, lo), own_excl = __shfl_sync(FULL, incl - n, lo);
      if (t < total) {
        const int p = own_first + (t - own_excl);
        const float4 pt = __ldg(G.p32 + p);
        const float dx = pt.x - qx, dy = pt.y - qy, dz = pt.z - qz;
        const float d2 = fmaf(dx, dx, fmaf(dy, dy, dz * dz));
        if (d2 < best || (d2 == best && bidx >= 0 && p < bidx)) {
          best = d2;
          bidx = p;
        }
      }
    }
    unsigned long long key = nn_key(best, bidx);
    for (int o = 16; o > 0; o >>= 1) {
      const unsigned long long k2 = __shfl_xor_sync(FULL, key, o);
      key = k2 < key ? k2 : key;
    }
    best = __uint_as_float((unsigned)(key >> 32));
    bidx = (int)(unsigned)(key & 0xffffffffu);
    if (stop) break;
  }
  return true;
}

// warp_nearest_list32 for two queries at once, one per half warp (lanes 0-15 and 16-31), each half
// scanning its query's list 32 entries at a time (two per lane), so a warp keeps two queries' chains
// of dependent loads in flight.  Every warp intrinsic runs on all 32 lanes; a half without work (no
// list, or its scan ended) takes part with empty values.  rng: the half's list range (x < 0: none,
// the half is left as it is); best / bidx: per half, the bound and candidate on entry (the same on
// the half's lanes), the result on return.  Same result as warp_nearest_list32.
__device__ __forceinline__ void halfwarp_list_nearest32(const PmGridDev& G, float qx, float qy, float qz, int2 rng, float& best,
                                                        int& bidx) {
  const unsigned FULL = 0xffffffffu;
  const int hl = threadIdx.x & 15;
  const float unit = G.cell32 * (1.0f / (float)PM_CL_UNITS);
  bool live = rng.x >= 0;  // the same on the half's lanes
  for (int base = 0; __ballot_sync(FULL, live) != 0; base += 32) {  // warp-uniform
    int2 pr0 = make_int2(0, 0), pr1 = make_int2(0, 0);
    bool beyond1 = true;  // the lane's second entry; on lane 15 of the half, the chunk's last
    if (live) {
      const int k0 = rng.x + base + hl, k1 = k0 + 16;
      const uint32_t e0 = k0 < rng.y ? __ldg(G.cl_ent + k0) : 0xffffffffu;
      const uint32_t e1 = k1 < rng.y ? __ldg(G.cl_ent + k1) : 0xffffffffu;
      const float l0 = (float)(e0 >> 24) * unit, l1 = (float)(e1 >> 24) * unit;
      const bool beyond0 = k0 >= rng.y || l0 * l0 * (1.0f - 1e-5f) >= best;
      beyond1 = k1 >= rng.y || l1 * l1 * (1.0f - 1e-5f) >= best;
      if (!beyond0) {
        const int o = (int)(e0 & 0xffffffu);
        const float4 lo = __ldg(G.cell_rec + 2 * o), hi = __ldg(G.cell_rec + 2 * o + 1);
        const float gx = gap32(qx, lo.x, hi.x), gy = gap32(qy, lo.y, hi.y), gz = gap32(qz, lo.z, hi.z);
        if (fmaf(gx, gx, fmaf(gy, gy, gz * gz)) < best) pr0 = make_int2(__float_as_int(lo.w), __float_as_int(hi.w));
      }
      if (!beyond1) {
        const int o = (int)(e1 & 0xffffffu);
        const float4 lo = __ldg(G.cell_rec + 2 * o), hi = __ldg(G.cell_rec + 2 * o + 1);
        const float gx = gap32(qx, lo.x, hi.x), gy = gap32(qy, lo.y, hi.y), gz = gap32(qz, lo.z, hi.z);
        if (fmaf(gx, gx, fmaf(gy, gy, gz * gz)) < best) pr1 = make_int2(__float_as_int(lo.w), __float_as_int(hi.w));
      }
    }
    const bool stop = __shfl_sync(FULL, beyond1 ? 1 : 0, 15, 16) != 0;
    // the points of the surviving cells, spread over the half's lanes
    const int n0 = pr0.y - pr0.x, n = n0 + (pr1.y - pr1.x);
    int incl = n;
    for (int o = 1; o < 16; o <<= 1) {
      const int t = __shfl_up_sync(FULL, incl, o, 16);
      if (hl >= o) incl += t;
    }
    const int total = __shfl_sync(FULL, incl, 15, 16);
    const int other = __shfl_xor_sync(FULL, total, 16);
    const int rounds = total > other ? total : other;  // warp-uniform
    for (int t0 = 0; t0 < rounds; t0 += 16) {
      const int t = t0 + hl;
      int lo = 0, hi = 15;  // owner: the first lane of the half whose inclusive count exceeds t
      for (int it = 0; it < 4; it++) {
        const int mid = (lo + hi) >> 1;
        if (__shfl_sync(FULL, incl, mid, 16) <= t) lo = mid + 1;
        else hi = mid;
      }
      const int own_excl = __shfl_sync(FULL, incl - n, lo, 16);
      const int own_n0 = __shfl_sync(FULL, n0, lo, 16);
      const int own_p0 = __shfl_sync(FULL, pr0.x, lo, 16), own_p1 = __shfl_sync(FULL, pr1.x, lo, 16);
      if (t < total) {
        const int off = t - own_excl;
        const int p = off < own_n0 ? own_p0 + off : own_p1 + (off - own_n0);
        const float4 pt = __ldg(G.p32 + p);
        const float dx = pt.x - qx, dy = pt.y - qy, dz = pt.z - qz;
        const float d2 = fmaf(dx, dx, fmaf(dy, dy, dz * dz));
        if (d2 < best || (d2 == best && bidx >= 0 && p < bidx)) {
          best = d2;
          bidx = p;
        }
      }
    }
    unsigned long long key = nn_key(best, bidx);
    for (int o = 8; o > 0; o >>= 1) {  // within the half
      const unsigned long long k2 = __shfl_xor_sync(FULL, key, o);
      key = k2 < key ? k2 : key;
    }
    best = __uint_as_float((unsigned)(key >> 32));
    bidx = (int)(unsigned)(key & 0xffffffffu);
    live = live && !stop;
  }
}

// Warp-cooperative bounded nearest neighbour (FP32): all 32 lanes call it with the same query
// (and the same optional starting candidate).
// Where q's fine cell has a cell list, the list answers (warp_nearest_list32).  Elsewhere: the
// block's candidate list, or the walk below.  Blocks are visited nearest-first, 32 offsets at a time, until the next offset's lower bound
// clears the current best; every block that may hold a point below the best is handed to all
// lanes, which split its occupied cells and test their points; the warp minimum is shared after
// every block.  Result: the exact minimum of the FP32 squared distances below maxd2 (among
// equal values the smallest sorted index), as grid_nearest32.
__device__ inline NNResult32 warp_nearest32(const PmGridDev& G, float qx, float qy, float qz, float maxd2, float init_d2 = INFINITY,
                                            int init_idx = -1, int2 list_rng = make_int2(-2, -2)) {
  const unsigned FULL = 0xffffffffu;
  const int lane = threadIdx.x & 31;
  NNResult32 r{maxd2, -1};
  if (G.n_points <= 0 || !isfinite(qx) || !isfinite(qy) || !isfinite(qz)) return r;  // as grid_nearest64
  // a known point (init_idx at init_d2, e.g. the nearest point of the query's field cell) starts the
  // walk with a tight bound
  float best = init_d2 < maxd2 ? init_d2 : maxd2;
  int bidx = init_d2 < maxd2 ? init_idx : -1;
  if (warp_nearest_list32(G, qx, qy, qz, best, bidx, list_rng)) {
    r.d2 = best;
    r.idx = bidx;
    return r;
  }
  const float reach = sqrtf(maxd2);
  const float blk = G.blk32;
  const float inv = G.inv_blk32;
  const float qa[3] = {qx, qy, qz};
  const float oa[3] = {G.o32[0], G.o32[1], G.o32[2]};
  const int nb[3] = {G.nbx, G.nby, G.nbz};
  int cb[3];
  bool inside = true;
  for (int a = 0; a < 3; a++) {
    const float f = floorf((qa[a] - oa[a]) * inv);
    if (!(f >= 0.f && f <= (float)(nb[a] - 1))) inside = false;
    cb[a] = !(f >= 0.f) ? 0 : (f > (float)(nb[a] - 1) ? nb[a] - 1 : (int)f);
  }
  auto process = [&](bool cand, int2 occ) {
    unsigned bal = __ballot_sync(FULL, cand);
    while (bal) {
      const int src = __ffs(bal) - 1;
      bal &= bal - 1;
      const int c0 = __shfl_sync(FULL, occ.x, src), c1 = __shfl_sync(FULL, occ.y, src);
      for (int c = c0 + lane; c < c1; c += 32) {
        const float4 lo = __ldg(G.cell_rec + 2 * c), hi = __ldg(G.cell_rec + 2 * c + 1);
        const float gx = gap32(qx, lo.x, hi.x), gy = gap32(qy, lo.y, hi.y), gz = gap32(qz, lo.z, hi.z);
        if (fmaf(gx, gx, fmaf(gy, gy, gz * gz)) >= best) continue;
        const int2 pr = make_int2(__float_as_int(lo.w), __float_as_int(hi.w));
        for (int p = pr.x; p < pr.y; p++) {
          const float4 pt = __ldg(G.p32 + p);
          const float dx = pt.x - qx, dy = pt.y - qy, dz = pt.z - qz;
          const float d2 = fmaf(dx, dx, fmaf(dy, dy, dz * dz));
          if (d2 < best || (d2 == best && bidx >= 0 && p < bidx)) {
            best = d2;
            bidx = p;
          }
        }
      }
      unsigned long long k = nn_key(best, bidx);
      for (int o = 16; o > 0; o >>= 1) {
        const unsigned long long k2 = __shfl_xor_sync(FULL, k, o);
        k = k2 < k ? k2 : k;
      }
      best = __uint_as_float((unsigned)(k >> 32));
      bidx = (int)(unsigned)(k & 0xffffffffu);
    }
  };
  if (inside && G.blk_list) {  // the block's candidate list covers every point within its reach
    const int b = cb[0] + nb[0] * (cb[1] + nb[1] * cb[2]);
    const int2 rng = __ldg(G.blk_list + b);
    if (rng.x >= 0 && sqrtf(best) <= __ldg(G.blk_reach + b)) {
      // 32 list entries at a time: the occupied cells of every entry whose box is below the best
      // are concatenated (warp scan of their counts) and split evenly across the lanes
      for (int base = rng.x; base < rng.y; base += 32) {
        const int k = base + lane;
        int2 occ = make_int2(0, 0);
        int n = 0;
        bool beyond = true;  // this entry, and (sorted) every later one, lies beyond the best
        if (k < rng.y) {  // the widened entry and its block's box: no dependent load
          const int4 e = __ldg(G.cand4 + k);
          const float4 lo = __ldg(G.cand_box + 2 * k), hi = __ldg(G.cand_box + 2 * k + 1);
          const float ed = __int_as_float(e.w);
          beyond = ed * ed * (1.0f - 1e-5f) >= best;
          if (!beyond) {
            occ = make_int2(e.x, e.y);
            const float gx = gap32(qx, lo.x, hi.x), gy = gap32(qy, lo.y, hi.y), gz = gap32(qz, lo.z, hi.z);
            if (fmaf(gx, gx, fmaf(gy, gy, gz * gz)) < best) n = occ.y - occ.x;
          }
        }
        const bool stop = __shfl_sync(FULL, beyond ? 1 : 0, 31) != 0;
        int incl = n;
        for (int o = 1; o < 32; o <<= 1) {
          const int t = __shfl_up_sync(FULL, incl, o);
          if (lane >= o) incl += t;
        }
        const int total = __shfl_sync(FULL, incl, 31);
        // up to 4 cells per lane per round: their box loads are independent, so they overlap;
        // then the point ranges of the surviving cells, then their points
        for (int t0 = 0; t0 < total; t0 += 128) {
          int cs[4];
#pragma unroll
          for (int j = 0; j < 4; j++) {
            const int t = t0 + 32 * j + lane;
            int lo = 0, hi = 31;  // owner: the first lane whose inclusive count exceeds t
            for (int it = 0; it < 5; it++) {
              const int mid = (lo + hi) >> 1;
              if (__shfl_sync(FULL, incl, mid) <= t) lo = mid + 1;
              else hi = mid;
            }
            const int own_first = __shfl_sync(FULL, occ.x, lo), own_excl = __shfl_sync(FULL, incl - n, lo);
            cs[j] = t < total ? own_first + (t - own_excl) : -1;
          }
          // box and point range of each cell in one record: one round trip instead of two
          int2 pr[4];
#pragma unroll
          for (int j = 0; j < 4; j++) {
            pr[j] = make_int2(0, 0);
            if (cs[j] >= 0) {
              const float4 lo = __ldg(G.cell_rec + 2 * cs[j]), hi = __ldg(G.cell_rec + 2 * cs[j] + 1);
              const float gx = gap32(qx, lo.x, hi.x), gy = gap32(qy, lo.y, hi.y), gz = gap32(qz, lo.z, hi.z);
              if (fmaf(gx, gx, fmaf(gy, gy, gz * gz)) < best) pr[j] = make_int2(__float_as_int(lo.w), __float_as_int(hi.w));
            }
          }
#pragma unroll
          for (int j = 0; j < 4; j++) {
            for (int p = pr[j].x; p < pr[j].y; p++) {
              const float4 pt = __ldg(G.p32 + p);
              const float dx = pt.x - qx, dy = pt.y - qy, dz = pt.z - qz;
              const float d2 = fmaf(dx, dx, fmaf(dy, dy, dz * dz));
              if (d2 < best || (d2 == best && bidx >= 0 && p < bidx)) {
                best = d2;
                bidx = p;
              }
            }
          }
        }
        unsigned long long key = nn_key(best, bidx);
        for (int o = 16; o > 0; o >>= 1) {
          const unsigned long long k2 = __shfl_xor_sync(FULL, key, o);
          key = k2 < key ? k2 : key;
        }
        best = __uint_as_float((unsigned)(key >> 32));
        bidx = (int)(unsigned)(key & 0xffffffffu);
        if (stop) break;
      }
      r.d2 = best;
      r.idx = bidx;
      return r;
    }
  }
  if (inside && reach < (float)(kOffR - 1) * blk) {
    // nearest-first over the sorted offsets; q lies in block cb up to FP32 rounding (4 um slack)
    for (int base = 0; base < kOffN; base += 32) {
      if (__ldg(c_off_lb + base) * blk - 4e-6f >= sqrtf(best)) break;
      const int k = base + lane;
      bool cand = false;
      int2 occ = make_int2(0, 0);
      if (k < kOffN) {
        const char4 o = __ldg(c_off + k);
        const int bx = cb[0] + o.x, by = cb[1] + o.y, bz = cb[2] + o.z;
        if (bx >= 0 && by >= 0 && bz >= 0 && bx < nb[0] && by < nb[1] && bz < nb[2]) {
          const int b = bx + nb[0] * (by + nb[1] * bz);
          occ = __ldg(reinterpret_cast<const int2*>(G.blk_occ) + b);
          cand = occ.x < occ.y && box_d2_32(G.blk_box + 6 * b, qx, qy, qz) < best;
        }
      }
      process(cand, occ);
    }
  } else {
    // the cube of blocks [q - reach, q + reach]
    int lo[3], hi[3];
    for (int a = 0; a < 3; a++) {
      // 1e-3 block of slack covers the FP32 rounding of the range against the FP64 assignment
      const float f0 = floorf((qa[a] - reach - oa[a]) * inv - 1e-3f), f1 = floorf((qa[a] + reach - oa[a]) * inv + 1e-3f);
      if (!(f1 >= 0.f) || !(f0 <= (float)(nb[a] - 1))) return r;  // also rejects NaN
      lo[a] = f0 < 0.f ? 0 : (int)f0;
      hi[a] = f1 > (float)(nb[a] - 1) ? nb[a] - 1 : (int)f1;
    }
    const int nx = hi[0] - lo[0] + 1, ny = hi[1] - lo[1] + 1, nz = hi[2] - lo[2] + 1;
    const int nblk = nx * ny * nz;
    for (int base = 0; base < nblk; base += 32) {
      const int i = base + lane;
      bool cand = false;
      int2 occ = make_int2(0, 0);
      if (i < nblk) {
        const int bx = lo[0] + i % nx;
        const int t = i / nx;
        const int by = lo[1] + t % ny, bz = lo[2] + t / ny;
        const int b = bx + nb[0] * (by + nb[1] * bz);
        occ = __ldg(reinterpret_cast<const int2*>(G.blk_occ) + b);
        cand = occ.x < occ.y && box_d2_32(G.blk_box + 6 * b, qx, qy, qz) < best;
      }
      process(cand, occ);
    }
  }
  r.d2 = best;
  r.idx = bidx;
  return r;
}

// Warp-cooperative exact FP64 nearest neighbour below maxd2: the minimum over points of
// fl(dx*dx + (dy*dy + dz*dz)) in FP64, as grid_nearest64.  The cube of blocks around q within
// sqrt(maxd2), one block of slack per side, is split across lanes; a candidate block's occupied
// cells are split across lanes and the warp minimum is shared after every block.
// The pruning runs in FP32 and only the points it cannot rule out reach FP64 (the FP64 pipe
// takes a whole warp instruction per operation, however few lanes are active): a block, cell or
// point is skipped when its FP32 distance from q exceeds the current best by more than the FP32
// error of both (t = 4e-7 (|q|_1 + |p|_1 max) + 4e-6 d, far above the rounding of the points,
// of q and of the distance arithmetic), so no point below the best is ever skipped.  hint: a
// point index whose distance starts the search (e.g. the FP32 nearest point), or -1.
__device__ inline NNResult64 warp_nearest64(const PmGridDev& G, const D3& q, double maxd2, int hint = -1) {
  const unsigned FULL = 0xffffffffu;
  const int lane = threadIdx.x & 31;
  NNResult64 r{maxd2, -1};
  if (G.n_points <= 0 || !(maxd2 > 0.0)) return r;
  double best = maxd2;
  int bidx = -1;
  if (hint >= 0 && hint < G.n_points) {
    const D3 d{G.px[hint] - q.x, G.py[hint] - q.y, G.pz[hint] - q.z};
    const double d2 = d.x * d.x + (d.y * d.y + d.z * d.z);
    if (d2 < best) {
      best = d2;
      bidx = hint;
    }
  }
  const float qx = (float)q.x, qy = (float)q.y, qz = (float)q.z;
  float pmax = 0.f;
  for (int a = 0; a < 3; a++) pmax += fmaxf(fabsf(G.box_lo32[a]), fabsf(G.box_hi32[a]));
  const float tabs = 4e-7f * (fabsf(qx) + fabsf(qy) + fabsf(qz) + pmax) + 1e-12f;
  // FP32 threshold on squared distances: anything above it is farther than the best
  auto thr = [&](double b) {
    const float sb = sqrtf((float)b) * (1.0f + 4e-6f) + tabs;
    return sb * sb * (1.0f + 1e-6f);
  };
  float t32 = thr(best);
  // warp minimum of (best, bidx); best >= 0, so its bits order like its value
  auto warp_min = [&]() {
    long long bb = __double_as_longlong(best);
    for (int o = 16; o > 0; o >>= 1) {
      const long long ob = __shfl_xor_sync(FULL, bb, o);
      const int oi = __shfl_xor_sync(FULL, bidx, o);
      if (ob < bb || (ob == bb && oi >= 0 && (bidx < 0 || oi < bidx))) {
        bb = ob;
        bidx = oi;
      }
    }
    best = __longlong_as_double(bb);
    t32 = thr(best);
  };
  // Where q's fine cell has a cell list (every occupied cell that can hold q's nearest point, nearest
  // first), the warp scans it 32 entries at a time: an entry whose stored lower bound reaches the
  // FP32 threshold ends the scan, the others are tested by their box, and the points of each
  // surviving cell are split over the lanes (FP32 prefilter, then the exact FP64 distance).
  int2 rng;
  if (cell_list_of(G, qx, qy, qz, rng)) {  // the same on every lane
    const float unit = G.cell32 * (1.0f / (float)PM_CL_UNITS);
    for (int base = rng.x; base < rng.y; base += 32) {  // warp-uniform
      const int k = base + lane;
      bool beyond = true;  // this entry, and (sorted) every later one, lies beyond the best
      int2 pr = make_int2(0, 0);
      if (k < rng.y) {
        const uint32_t e = __ldg(G.cl_ent + k);
        const float lbd = (float)(e >> 24) * unit;
        beyond = lbd * lbd * (1.0f - 1e-5f) >= t32;
        if (!beyond) {
          const int o = (int)(e & 0xffffffu);
          const float4 lo = __ldg(G.cell_rec + 2 * o), hi = __ldg(G.cell_rec + 2 * o + 1);
          const float gx = gap32(qx, lo.x, hi.x), gy = gap32(qy, lo.y, hi.y), gz = gap32(qz, lo.z, hi.z);
          if (!(fmaf(gx, gx, fmaf(gy, gy, gz * gz)) > t32)) pr = make_int2(__float_as_int(lo.w), __float_as_int(hi.w));
        }
      }
      const bool stop = __shfl_sync(FULL, beyond ? 1 : 0, 31) != 0;
      for (unsigned bal = __ballot_sync(FULL, pr.y > pr.x); bal != 0; bal &= bal - 1) {  // warp-uniform
        const int src = __ffs(bal) - 1;
        const int p0 = __shfl_sync(FULL, pr.x, src), p1 = __shfl_sync(FULL, pr.y, src);
        for (int pi = p0 + lane; pi < p1; pi += 32) {
          const float4 pt = __ldg(G.p32 + pi);
          const float ex = pt.x - qx, ey = pt.y - qy, ez = pt.z - qz;
          if (fmaf(ex, ex, fmaf(ey, ey, ez * ez)) > t32) continue;
          const D3 d{G.px[pi] - q.x, G.py[pi] - q.y, G.pz[pi] - q.z};
          const double d2 = d.x * d.x + (d.y * d.y + d.z * d.z);
          if (d2 < best || (d2 == best && bidx >= 0 && pi < bidx)) {
            best = d2;
            bidx = pi;
          }
        }
      }
      warp_min();
      if (stop) break;
    }
    r.d2 = best;
    r.idx = bidx;
    return r;
  }
  const float reach = sqrtf((float)maxd2) * (1.0f + 1e-6f);
  const float qa[3] = {qx, qy, qz};
  const int nb[3] = {G.nbx, G.nby, G.nbz};
  int lo[3], hi[3];
  for (int a = 0; a < 3; a++) {
    const float f0 = floorf((qa[a] - reach - G.o32[a]) * G.inv_blk32) - 1.0f;
    const float f1 = floorf((qa[a] + reach - G.o32[a]) * G.inv_blk32) + 1.0f;
    if (!(f1 >= 0.f) || !(f0 <= (float)(nb[a] - 1))) {  // also rejects NaN
      r.d2 = best;
      r.idx = bidx;
      return r;
    }
    lo[a] = f0 < 0.f ? 0 : (int)f0;
    hi[a] = f1 > (float)(nb[a] - 1) ? nb[a] - 1 : (int)f1;
  }
  const int nx = hi[0] - lo[0] + 1, ny = hi[1] - lo[1] + 1, nz = hi[2] - lo[2] + 1;
  const int nblk = nx * ny * nz;
  for (int base = 0; base < nblk; base += 32) {
    const int i = base + lane;
    bool cand = false;
    int2 occ = make_int2(0, 0);
    if (i < nblk) {
      const int bx = lo[0] + i % nx;
      const int t = i / nx;
      const int by = lo[1] + t % ny, bz = lo[2] + t / ny;
      const int b = bx + nb[0] * (by + nb[1] * bz);
      occ = __ldg(reinterpret_cast<const int2*>(G.blk_occ) + b);
      cand = occ.x < occ.y && !(box_d2_32(G.blk_box + 6 * b, qx, qy, qz) > t32);
    }
    unsigned bal = __ballot_sync(FULL, cand);
    while (bal) {
      const int src = __ffs(bal) - 1;
      bal &= bal - 1;
      const int c0 = __shfl_sync(FULL, occ.x, src), c1 = __shfl_sync(FULL, occ.y, src);
      for (int c = c0 + lane; c < c1; c += 32) {
        if (box_d2_32(G.cell_box + 6 * c, qx, qy, qz) > t32) continue;
        const int2 pr = __ldg(reinterpret_cast<const int2*>(G.cell_pts) + c);
        for (int p = pr.x; p < pr.y; p++) {
          const float4 pt = __ldg(G.p32 + p);
          const float ex = pt.x - qx, ey = pt.y - qy, ez = pt.z - qz;
          if (fmaf(ex, ex, fmaf(ey, ey, ez * ez)) > t32) continue;
          const D3 d{G.px[p] - q.x, G.py[p] - q.y, G.pz[p] - q.z};
          const double d2 = d.x * d.x + (d.y * d.y + d.z * d.z);
          if (d2 < best || (d2 == best && bidx >= 0 && p < bidx)) {
            best = d2;
            bidx = p;
            t32 = thr(best);
          }
        }
      }
      warp_min();
    }
  }
  r.d2 = best;
  r.idx = bidx;
  return r;
}

// is_outside(p, r) of a point cloud (primitive_sdf.hpp:597-603) with the warp search: only
// whether a point lies within r + radius matters (see prim_outside).  Warp-uniform arguments.
__device__ __forceinline__ bool cloud_outside_warp(const PmPrim& P, const PmGridDev* clouds, const D3& p, double r, int* near,
                                                   int hint = -1) {
  const double reach = (r + P.a) * (1.0 + 1e-12) + 1e-12;
  const NNResult64 nn = warp_nearest64(clouds[P.cloud], p, reach * reach, hint);
  if (near) *near = nn.idx;
  if (nn.idx < 0) return true;
  return sqrt(nn.d2) - P.a > r;
}

// Starting candidate of a warp search, in two steps so that the loads can be issued early: the field
// record (nearest point and index) of one of the 8 fine-cell centres around q on lanes 0-7 (index -1
// elsewhere and outside the grid), and q's own cell-list range on lane 8 (int bits in x, y; -1 none);
// then the best of the 8 shared by the warp ((INFINITY, -1) if none) and the list range.
// sub: the lane's position in its query's group of lanes (the lane itself for a whole warp; 0-15 for
// a half warp).
__device__ __forceinline__ float4 field_corner_record(const PmGridDev& G, float qx, float qy, float qz, int sub) {
  const int lane = sub;
  float4 rec = make_float4(__int_as_float(-1), __int_as_float(-1), 0.f, __int_as_float(-1));
  if (lane < 8 && G.n_points > 0) {
    const float inv = G.inv_cell32;
    const float qa[3] = {qx, qy, qz};
    const int nc[3] = {G.nbx * PM_GRID_B, G.nby * PM_GRID_B, G.nbz * PM_GRID_B};
    int cc[3];
    bool ok = true;
    for (int a = 0; a < 3; a++) {
      const float t = floorf((qa[a] - G.o32[a]) * inv - 0.5f) + (float)((lane >> a) & 1);
      ok = ok && t >= 0.f && t <= (float)(nc[a] - 1);
      cc[a] = ok ? (int)t : 0;
    }
    if (ok) rec = __ldg(G.cell_np + cc[0] + nc[0] * (cc[1] + (int64_t)nc[1] * cc[2]));
  } else if (lane == 8 && G.n_points > 0) {
    int2 rng;
    if (cell_list_of(G, qx, qy, qz, rng)) rec = make_float4(__int_as_float(rng.x), __int_as_float(rng.y), 0.f, __int_as_float(-1));
  }
  return rec;
}
struct FieldStart {
  NNResult32 nn;  // the best of the 8 corner records
  int2 rng;       // q's cell-list range (-1: none)
};
// width: 32 (one query per warp) or 16 (one per half warp; every lane calls it).
__device__ __forceinline__ FieldStart field_corner_candidate(const float4& rec, float qx, float qy, float qz, int width = 32) {
  const unsigned FULL = 0xffffffffu;
  const int lane = threadIdx.x & (width - 1);
  const int idx = __float_as_int(rec.w);
  unsigned long long key = ~0ull;
  if (lane < 8 && idx >= 0) {  // the FP32 expression of every walk (point_d2_32)
    const float dx = rec.x - qx, dy = rec.y - qy, dz = rec.z - qz;
    key = nn_key(fmaf(dx, dx, fmaf(dy, dy, dz * dz)), idx);
  }
  for (int o = 4; o > 0; o >>= 1) {
    const unsigned long long k2 = __shfl_xor_sync(FULL, key, o);
    key = k2 < key ? k2 : key;
  }
  key = __shfl_sync(FULL, key, 0, width);
  const int rx = __shfl_sync(FULL, __float_as_int(rec.x), 8, width), ry = __shfl_sync(FULL, __float_as_int(rec.y), 8, width);
  FieldStart f{{INFINITY, -1}, make_int2(rx, ry)};
  if (key != ~0ull) {
    f.nn.d2 = __uint_as_float((unsigned)(key >> 32));
    f.nn.idx = (int)(unsigned)(key & 0xffffffffu);
  }
  return f;
}

__device__ __forceinline__ int f2o(float f) {
  const int i = __float_as_int(f);
  return i >= 0 ? i : i ^ 0x7fffffff;
}
__device__ __forceinline__ float o2f(int i) { return __int_as_float(i >= 0 ? i : i ^ 0x7fffffff); }

template <class Src>
__device__ __forceinline__ void push_item(const Scratch& s, const Src& src, int64_t b, int kind_x, int i, int j) {
  if (b > 0x7fffffffLL) {  // the queue stores 32-bit indices: beyond them, the full FP64 check decides
    s.overflow[src.overflow_slot(b)] = 1;
    return;
  }
  unsigned int k = atomicAdd(s.count, 1u);
  if (k < s.cap) {
    s.items[k] = make_int4((int)b, kind_x, i, j);
  } else {
    s.overflow[src.overflow_slot(b)] = 1;
  }
}

struct Smem {
  double* qbuf;  // generated configurations (edges)
  int2* hq;      // hard cloud queries: (cfg << 16 | sphere, primitive)
  unsigned char* fkl;  // the two-thread FK's slot lists: [0, 64) phase 0, [64, 128) and [128, 192) the
                       // two threads of phase 1; fkn[0..2] their lengths
  int* fkn;
  int* hq_n;     // [0] pushed, [1] popped
  int* sdist;    // per (cfg, sphere): running minimum signed distance, order-preserving int
  float* pose;   // [cfg][slot][kPoseF]
  SlotF* slot;
  float* base8;  // fixed base pose: q xyzw, t xyz
  SphereF* sph;
  GroupF* grp;
  PrimF* prm;
  int2* pairs;
  int* flags;
  unsigned* cull;  // [cfg][group]: bit p set -> primitive p certainly clears the whole group
};

// Where a block's configurations come from and where their outcomes go.
struct CfgSource {  // a batch of configurations q[B x q_dim]
  const double* q;
  int64_t B;
  uint8_t* out;
  PmLinkBounds bnd;  // link-position bounds checked with the collision terms (composite constraint)
  __device__ const double* cfg(const PmTablesHdr* T, int64_t i, double*) const { return q + i * T->q_dim; }
  __device__ bool pre_skip(int64_t) const { return false; }     // before the fast pass: nothing known
  __device__ bool skip(int64_t i) const { return out[i] == 0; }  // after it: already invalid
  __device__ void fail(int64_t i) const { out[i] = 0; }
  __device__ void done(int64_t i, bool failed) const { out[i] = failed ? 0 : 1; }
  __device__ int64_t overflow_slot(int64_t i) const { return i; }
  __device__ int64_t n_overflow_slots() const { return B; }
  __device__ void full_check(const TView& v, const double* state, int64_t i, double*) const {
    out[i] = is_valid_cfg(v, state, q + i * v.T->q_dim, bnd) ? 1 : 0;
  }
};

// Edges of checkMotion flattened into waypoints: edge e owns waypoints [off[e], off[e] + n[e]);
// waypoint k of an edge is s2 for k = 0, then the interior points in the reference's visiting
// order (motion_validator.cpp:45-78).
struct EdgeSource {
  const double* s1;
  const double* s2;
  const int64_t* off;
  const int32_t* n;
  const double* sr;
  const int16_t* seq;
  int64_t E;
  uint8_t* valid;  // per edge, 1 until a waypoint is found colliding
  PmLinkBounds bnd;  // link-position bounds checked at every waypoint (composite constraint)
  __device__ int64_t edge_of(int64_t w) const {
    int64_t lo = 0, hi = E - 1;
    while (lo < hi) {
      int64_t mid = (lo + hi + 1) >> 1;
      if (off[mid] <= w) lo = mid; else hi = mid - 1;
    }
    return lo;
  }
  __device__ const double* cfg(const PmTablesHdr* T, int64_t w, double* buf) const {
    const int64_t e = edge_of(w);
    const int64_t k = w - off[e];
    const int d = T->q_dim;
    const double* a = s1 + e * d;
    const double* b = s2 + e * d;
    if (k == 0) return b;
    const double r = sr[e];
    const unsigned long long n_test = (unsigned long long)n[e] + 1;  // floor(1 / r) + 2, from k_edge_setup
    double t;
    if (n_test < 129) {
      t = (double)seq[(n_test - 1) * 128 + (k + 1)] * r;
    } else {
      t = (double)k * r;
    }
    for (int i = 0; i < d; i++) buf[i] = a[i] + (b[i] - a[i]) * t;
    return buf;
  }
  __device__ bool pre_skip(int64_t w) const { return valid[edge_of(w)] == 0; }
  __device__ bool skip(int64_t w) const { return valid[edge_of(w)] == 0; }
  __device__ void fail(int64_t w) const { valid[edge_of(w)] = 0; }
  __device__ void done(int64_t w, bool failed) const {
    if (failed) valid[edge_of(w)] = 0;
  }
  __device__ int64_t overflow_slot(int64_t w) const { return edge_of(w); }
  __device__ int64_t n_overflow_slots() const { return E; }
  // every waypoint of edge e in the plain FP64 method
  __device__ void full_check(const TView& v, const double* state, int64_t e, double* buf) const {
    bool ok = true;
    for (int64_t w = off[e]; w < off[e] + n[e] && ok; w++) ok = is_valid_cfg(v, state, cfg(v.T, w, buf), bnd);
    if (!ok) valid[e] = 0;
  }
};

// Phases 1-3 for the configurations [c0, c0 + ncfg) of a source.  qbuf holds CPB * q_dim
// doubles of shared memory for generated configurations.
template <int CPB, class Src>
__device__ void fast_block(const TView& v, const Smem& sm, const double* __restrict__ state, const Src& src, int64_t c0, int ncfg,
                           float* __restrict__ dist32, float cutoff, const Scratch& scr, double* qbuf) {
  const PmTablesHdr* T = v.T;
  const int ns = T->n_spheres, ng = T->n_groups, np = T->n_prims, npr = T->n_pairs, nsl = T->n_slots;
  const int tid = threadIdx.x;
  // ---- 1. FK (FP32, with error bounds) -> shared memory, two threads per configuration (threads 2c
  //         and 2c + 1): the trunk of the slot tree by the first, then one subtree set each (the
  //         host's split); the configuration goes to qbuf so that both threads read it
  {
    const int fc = tid >> 1, fth = tid & 1;
    const int qd = T->q_dim;
    const bool taylor = T->base_type == PM_BASE_FIXED;
    float* P = sm.pose + (size_t)fc * nsl * kPoseF;
    if (fth == 0 && fc < CPB) {
      int fl = 0;
      if (fc < ncfg) {
        if (src.pre_skip(c0 + fc)) {
          fl = FLAG_FAIL | 2;  // already known invalid: no work
        } else {
          double* qb = qbuf + fc * qd;
          const double* qc = src.cfg(T, c0 + fc, qb);
          bool finite = true;
          for (int i = 0; i < qd; i++) {
            const double x = qc[i];
            finite = finite && finite64(x);
            qb[i] = x;
          }
          if (finite) {
            fk32(sm.slot, sm.fkn[0], sm.base8, T->base_type, T->n_ctrl, qb, taylor, P, 1, sm.fkl);
          } else {
            // a NaN or infinite coordinate makes every FP32 bound NaN, and no decision would be taken:
            // the exact FP64 check of the recheck kernel decides, as for an overflowing queue
            fl = 2;
            scr.overflow[src.overflow_slot(c0 + fc)] = 1;
          }
        }
      }
      sm.flags[fc] = fl;
    }
    __syncthreads();
    if (fc < ncfg && !(sm.flags[fc] & 2))
      fk32(sm.slot, sm.fkn[1 + fth], sm.base8, T->base_type, T->n_ctrl, qbuf + fc * qd, taylor, P, 1, sm.fkl + (1 + fth) * PM_MAX_SLOTS);
  }
  __syncthreads();
  const bool want_dist = dist32 != nullptr;
  // ---- 1b. link-position bounds of a composite constraint (LinkPositionBoundCst::is_valid_dirty,
  //          primitive_link_position_bound.cpp:69-79): the link's FP32 world position and its FK
  //          error bound decide; an undecided bound goes to the FP64 recheck.  A failed bound marks
  //          the configuration before the sphere tasks, which then skip it (validity mode).
  for (int t = tid, nb = src.bnd.n; t < ncfg * nb; t += blockDim.x) {
    const int c = t / nb, k = t - c * nb;
    if (sm.flags[c] & 2) continue;
    const PmPoseTerm& b = src.bnd.t[k];
    const float* P = sm.pose + ((size_t)c * nsl + b.slot) * kPoseF;
    const float x = P[9 + b.axis];
    const float lo = (float)b.lb, hi = (float)b.ub;
    // the FK error bound, plus the rounding of the bounds to FP32 and of the comparison
    const float m = P[12] + margin32(fabsf(x) + (b.has_lb ? fabsf(lo) : 0.f) + (b.has_ub ? fabsf(hi) : 0.f));
    const bool fail = (b.has_lb && x + m < lo) || (b.has_ub && x - m > hi);
    if (fail) atomicOr(&sm.flags[c], FLAG_FAIL);
    else if ((b.has_lb && x - m <= lo) || (b.has_ub && x + m >= hi)) push_item(scr, src, c0 + c, -1 - k, 0, 0);
  }
  // ---- 2. group culling against each primitive
  for (int t = tid; t < ncfg * ng; t += blockDim.x) {
    const int c = t / ng, gi = t - c * ng;
    if (sm.flags[c] & 2) continue;
    const GroupF& G = sm.grp[gi];
    const float* P = sm.pose + ((size_t)c * nsl + G.slot) * kPoseF;
    float3 gc = xf(P, G.rel[0], G.rel[1], G.rel[2]);
    const float ekg = P[12] + P[13] * G.gn;  // FK error bound of the group centre
    unsigned mask = 0;
    const int npc = np < 32 ? np : 32;
    for (int p = 0; p < npc; p++) {
      float g, sd, mag;
      const PrimF& P = sm.prm[p];
      if (P.kind == PM_SDF_CLOUD) {  // the nearest-point field bounds the cloud from below
        const float lb = grid_field_lb16(v.C[P.cloud], gc.x, gc.y, gc.z);
        g = lb - P.a - G.radius;
        mag = fabsf(gc.x) + fabsf(gc.y) + fabsf(gc.z) + lb;
      } else {
        clearance(P, v.C, gc.x, gc.y, gc.z, G.radius, G.tiny, 0.f, g, sd, mag);
      }
      if (g > margin32(mag) + ekg + (want_dist ? cutoff : 0.f)) mask |= 1u << p;
    }
    sm.cull[c * ng + gi] = mask;
  }
  __syncthreads();
  // ---- 3a. sphere tasks (primitives in-thread; cloud queries near the cloud are queued) and
  //          self-pair tasks
  if (tid == 0) {
    sm.hq_n[0] = 0;
    sm.hq_n[1] = 0;
  }
  __syncthreads();
  const int hq_cap = T->n_clouds > 0 ? CPB * ns : 0;
  // Sphere tasks in warp rows of 32 / ST configurations (fastest) x ST spheres; ST = 2^stl is the
  // sphere tile (autotuned), at least 32 / CPB so that a row holds every configuration once.  A small
  // tile puts the same sphere on neighbouring lanes (shared records); a large one keeps a
  // configuration's neighbouring spheres, and so their field cells, on one warp.  Pair tasks
  // follow, numbered with the configuration fastest.  CPB is a power of two: no division.
  constexpr int cpb_l = CPB == 16 ? 4 : (CPB == 32 ? 5 : (CPB == 64 ? 6 : 7));
  const int stl = max(min(scr.st_log2, 5), cpb_l >= 5 ? 0 : 5 - cpb_l);
  const int rl = 5 - stl, ncb_l = cpb_l - rl;  // configurations per row, rows per sphere tile (log2)
  const int n_sph_tasks = (((ns + (1 << stl) - 1) >> stl) << ncb_l) << 5;
  const int n_tasks = n_sph_tasks + npr * CPB;
  const unsigned all_culled = np >= 32 ? 0xffffffffu : ((1u << np) - 1u);
  // one sphere of one configuration: primitives in-thread, cloud queries near the cloud queued
  auto sphere_task = [&](int si, int c) {
    if (c >= ncfg || (sm.flags[c] & 2)) return;
    const SphereF S = sm.sph[si];
    const GroupF& G = sm.grp[S.group];
    const bool check = !G.only_self && np > 0;
    if (!want_dist && (!check || (sm.flags[c] & FLAG_FAIL))) return;
    const unsigned cm = sm.cull[c * ng + S.group];
    if (np <= 32 && cm == all_culled) {  // the group sphere clears every primitive (by the cutoff too)
      if (want_dist) sm.sdist[c * ns + si] = f2o(cutoff);
      return;
    }
    const float* P = sm.pose + ((size_t)c * nsl + G.slot) * kPoseF;
    const float3 sc = xf(P, S.x, S.y, S.z);
    const float ek = P[12] + P[13] * S.sn;  // FK error bound of the sphere centre
    float sdmin = cutoff;
    int fail = 0;
    const float m = margin32(4.0f + fabsf(sc.x) + fabsf(sc.y) + fabsf(sc.z)) + ek;
    for (int p = 0; p < np; p++) {
      if (p < 32 && ((cm >> p) & 1u)) continue;
      const PrimF& Pr = sm.prm[p];
      float g, sd, mag;
      if (Pr.kind == PM_SDF_CLOUD) {
        const PmGridDev& Gc = v.C[Pr.cloud];
        // the field's 16-bit bound first (one 2-byte load); the nearest point only where the
        // validity-only shortcut below can use it
        const float lb = grid_field_lb16(Gc, sc.x, sc.y, sc.z);
        const float qmag = fabsf(sc.x) + fabsf(sc.y) + fabsf(sc.z);
        if (lb - Pr.a - S.r > margin32(qmag + lb) + ek + (want_dist ? cutoff : 0.f)) continue;
        const FieldLB fb = !want_dist && check ? grid_field32(Gc, sc.x, sc.y, sc.z, true) : FieldLB{lb, -1, make_float4(0.f, 0.f, 0.f, 0.f)};
        if (!want_dist && check && fb.idx >= 0) {
          // the centre's nearest point is a real point: if it is certainly within reach, the
          // sphere collides and no search is needed
          const float ex = fb.np.x - sc.x, ey = fb.np.y - sc.y, ez = fb.np.z - sc.z;
          const float ub = sqrtf(fmaf(ex, ex, fmaf(ey, ey, ez * ez)));
          if (ub - Pr.a - S.r < -(margin32(qmag + ub) + ek)) {
            fail = 1;
            break;
          }
        }
        const int k = atomicAdd(&sm.hq_n[0], 1);
        if (k < hq_cap) {
          sm.hq[k] = make_int2(c << 16 | si, p);
          continue;
        }
        clearance(Pr, v.C, sc.x, sc.y, sc.z, S.r, S.tiny, want_dist ? m + cutoff : m, g, sd, mag);
      } else {
        clearance(Pr, v.C, sc.x, sc.y, sc.z, S.r, S.tiny, 0.f, g, sd, mag);
      }
      sdmin = fminf(sdmin, sd);
      if (!check) continue;
      const float mm = margin32(mag) + ek;
      if (g < -mm) {
        fail = 1;
        if (!want_dist) break;
      } else if (g <= mm) {
        push_item(scr, src, c0 + c, p << 1, si, -1);
      }
    }
    if (fail) atomicOr(&sm.flags[c], FLAG_FAIL);
    if (want_dist) sm.sdist[c * ns + si] = f2o(sdmin);
  };
  // Self pairs: each lane tests its (configuration, group pair) by the group spheres; the warp then
  // takes the surviving pairs one at a time, 32 sphere pairs per step (rows of 8 x 4), so a rare
  // survivor does not hold 31 idle lanes for its whole sphere-pair loop.
  const unsigned FULL = 0xffffffffu;
  const int lane = tid & 31;
  for (int t0 = tid & ~31; t0 < n_tasks; t0 += blockDim.x) {  // warp-uniform
    const int t = t0 + lane;
    int hit_pi = -1, hit_c = 0;
    if (t < n_sph_tasks) {
      const int w = t >> 5, l = t & 31;
      const int c = ((w & ((1 << ncb_l) - 1)) << rl) + (l & ((1 << rl) - 1));
      const int si = ((w >> ncb_l) << stl) + (l >> rl);
      if (si < ns) sphere_task(si, c);
    } else if (t < n_tasks) {
      const int u = t - n_sph_tasks;
      const int pi = u / CPB, c = u % CPB;
      if (c < ncfg && !(sm.flags[c] & (FLAG_FAIL | 2))) {
        const int2 pr = sm.pairs[pi];
        const GroupF& G1 = sm.grp[pr.x];
        const GroupF& G2 = sm.grp[pr.y];
        const float* P1 = sm.pose + ((size_t)c * nsl + G1.slot) * kPoseF;
        const float* P2 = sm.pose + ((size_t)c * nsl + G2.slot) * kPoseF;
        const float3 a = xf(P1, G1.rel[0], G1.rel[1], G1.rel[2]);
        const float3 bb = xf(P2, G2.rel[0], G2.rel[1], G2.rel[2]);
        const float ddx = a.x - bb.x, ddy = a.y - bb.y, ddz = a.z - bb.z;
        const float gmag = fabsf(a.x) + fabsf(a.y) + fabsf(a.z) + fabsf(bb.x) + fabsf(bb.y) + fabsf(bb.z);
        if (!(sqrtf(fmaf(ddx, ddx, fmaf(ddy, ddy, ddz * ddz))) - (G1.radius + G2.radius) >
              2.0f * margin32(gmag) + P1[12] + P1[13] * G1.gn + P2[12] + P2[13] * G2.gn)) {
          hit_pi = pi;
          hit_c = c;
        }
      }
    }
    unsigned pend = __ballot_sync(FULL, hit_pi >= 0);
    while (pend) {
      const int src_lane = __ffs(pend) - 1;
      pend &= pend - 1;
      const int pi = __shfl_sync(FULL, hit_pi, src_lane), c = __shfl_sync(FULL, hit_c, src_lane);
      const int2 pr = sm.pairs[pi];
      const GroupF& G1 = sm.grp[pr.x];
      const GroupF& G2 = sm.grp[pr.y];
      const float* P1 = sm.pose + ((size_t)c * nsl + G1.slot) * kPoseF;
      const float* P2 = sm.pose + ((size_t)c * nsl + G2.slot) * kPoseF;
      int fail = 0;
      for (int jb = 0; jb < G2.count; jb += 8) {
        const int j = jb + (lane & 7);
        for (int ib = 0; ib < G1.count; ib += 4) {
          const int i = ib + (lane >> 3);
          if (i < G1.count && j < G2.count) {
            const SphereF Si = sm.sph[G1.begin + i];
            const SphereF Sj = sm.sph[G2.begin + j];
            const float3 ci = xf(P1, Si.x, Si.y, Si.z);
            const float3 cj = xf(P2, Sj.x, Sj.y, Sj.z);
            const float ex = ci.x - cj.x, ey = ci.y - cj.y, ez = ci.z - cj.z;
            const float g = sqrtf(fmaf(ex, ex, fmaf(ey, ey, ez * ez))) - (Si.r + Sj.r);
            const float mm = 2.0f * margin32(fabsf(ci.x) + fabsf(ci.y) + fabsf(ci.z) + fabsf(cj.x) + fabsf(cj.y) + fabsf(cj.z)) +
                             P1[12] + P1[13] * Si.sn + P2[12] + P2[13] * Sj.sn;
            if (g < -mm) fail = 1;
            else if (g <= mm) push_item(scr, src, c0 + c, (pi << 1) | 1, G1.begin + i, G2.begin + j);
          }
        }
        if (__any_sync(FULL, fail)) break;
      }
      if (fail) atomicOr(&sm.flags[c], FLAG_FAIL);
    }
  }
  __syncthreads();
  // ---- 3b. queued cloud queries, one warp per query; the next query's field records are read
  //          before the current query's walk, so their latency hides behind it
  {
    const int lane = tid & 31;
    const int nq = min(sm.hq_n[0], hq_cap);
    if (want_dist && scr.hq != nullptr && nq > 0) {  // block-uniform
      // with distances the queries go to k_hard_queries, which answers them without this block's
      // barriers; what does not fit in the global queue is answered here below
      if (tid == 0) {
        const unsigned long long base = atomicAdd(scr.hq_count, (unsigned long long)nq);
        const long long room = base >= scr.hq_cap ? 0 : (long long)scr.hq_cap - (long long)base;
        sm.hq_n[2] = room > 0 ? (int)base : 0;  // base < hq_cap whenever an entry goes out
        sm.hq_n[1] = room >= nq ? nq : (int)room;  // the local loop starts past these
      }
      __syncthreads();
      const unsigned base = (unsigned)sm.hq_n[2];
      const int n_out = sm.hq_n[1];
      for (int k = tid; k < n_out; k += blockDim.x) {
        const int2 e = sm.hq[k];
        const int c = e.x >> 16, si = e.x & 0xffff;
        const SphereF S = sm.sph[si];
        const GroupF& G = sm.grp[S.group];
        const PrimF& Pr = sm.prm[e.y];
        const float* P = sm.pose + ((size_t)c * nsl + G.slot) * kPoseF;
        const float3 sc = xf(P, S.x, S.y, S.z);
        const float ek = P[12] + P[13] * S.sn;
        const float m = margin32(4.0f + fabsf(sc.x) + fabsf(sc.y) + fabsf(sc.z)) + ek;
        const float reach = Pr.a + S.r + (m + cutoff);
        HardQuery h;
        h.a = make_float4(sc.x, sc.y, sc.z, reach);
        h.b = make_int4((int)(c0 + c), si | (e.y << 16) | (G.only_self ? 0 : (int)0x80000000u), __float_as_int(ek), 0);
        scr.hq[base + k] = h;
      }
      // the pops below advance hq_n[1]: every thread reads n_out (above) before any warp pops
      __syncthreads();
    }
    auto pop = [&]() {
      int k = 0;
      if (lane == 0) k = atomicAdd(&sm.hq_n[1], 1);
      return __shfl_sync(FULL, k, 0);
    };
    auto centre = [&](int k) {  // the queried sphere's centre
      const int2 e = sm.hq[k];
      const int c = e.x >> 16, si = e.x & 0xffff;
      const SphereF S = sm.sph[si];
      const float* P = sm.pose + ((size_t)c * nsl + sm.grp[S.group].slot) * kPoseF;
      return xf(P, S.x, S.y, S.z);
    };
    int k = pop();
    float4 rec = make_float4(__int_as_float(-1), __int_as_float(-1), 0.f, __int_as_float(-1));
    if (k < nq) {
      const float3 q = centre(k);
      rec = field_corner_record(v.C[sm.prm[sm.hq[k].y].cloud], q.x, q.y, q.z, lane);
    }
    while (k < nq) {
      const int kn = pop();
      float4 rec_n = make_float4(__int_as_float(-1), __int_as_float(-1), 0.f, __int_as_float(-1));
      if (kn < nq) {
        const float3 q = centre(kn);
        rec_n = field_corner_record(v.C[sm.prm[sm.hq[kn].y].cloud], q.x, q.y, q.z, lane);
      }
      const int2 e = sm.hq[k];
      const int c = e.x >> 16, si = e.x & 0xffff;
      const SphereF S = sm.sph[si];
      const GroupF& G = sm.grp[S.group];
      const bool check = !G.only_self;
      // warp-uniform: flags change under other warps, so lane 0 decides for the warp
      const int done_c = __shfl_sync(FULL, (!want_dist && (sm.flags[c] & FLAG_FAIL)) ? 1 : 0, 0);
      if (!done_c) {
        const PrimF& Pr = sm.prm[e.y];
        const float* P = sm.pose + ((size_t)c * nsl + G.slot) * kPoseF;
        const float3 sc = xf(P, S.x, S.y, S.z);
        const float ek = P[12] + P[13] * S.sn;
        const float m = margin32(4.0f + fabsf(sc.x) + fabsf(sc.y) + fabsf(sc.z)) + ek;
        const float reach = Pr.a + S.r + (want_dist ? m + cutoff : m);
        const PmGridDev& Gc = v.C[Pr.cloud];
        const FieldStart start = field_corner_candidate(rec, sc.x, sc.y, sc.z);
        const NNResult32 nn = warp_nearest32(Gc, sc.x, sc.y, sc.z, reach * reach, start.nn.d2, start.nn.idx, start.rng);
        if (lane == 0) {
          float g, sd, mag;
          if (nn.idx < 0) {
            g = reach - Pr.a - S.r;
            sd = 3.0e38f;
            mag = fabsf(sc.x) + fabsf(sc.y) + fabsf(sc.z);
          } else {
            const float d = sqrtf(nn.d2);
            g = d - Pr.a - S.r;
            sd = g;
            mag = fabsf(sc.x) + fabsf(sc.y) + fabsf(sc.z) + d;
          }
          if (want_dist) atomicMin(&sm.sdist[c * ns + si], f2o(sd));
          if (check) {
            const float mm = margin32(mag) + ek;
            if (g < -mm) {
              atomicOr(&sm.flags[c], FLAG_FAIL);
            } else if (g <= mm) {
              push_item(scr, src, c0 + c, e.y << 1, si, nn.idx);
            }
          }
        }
      }
      k = kn;
      rec = rec_n;
    }
  }
  __syncthreads();
  if (want_dist)
    for (int t = tid; t < ncfg * ns; t += blockDim.x) {  // sdist is [cfg][sphere]
      const int c = t / ns;
      // a configuration left to the exact check (non-finite coordinates) has no FP32 distances
      dist32[c0 * ns + t] = (sm.flags[c] & 2) && !(sm.flags[c] & FLAG_FAIL) ? __int_as_float(0x7fc00000) : o2f(sm.sdist[t]);
    }
  __syncthreads();
  if (tid < ncfg && !(sm.flags[tid] & 2)) src.done(c0 + tid, (sm.flags[tid] & FLAG_FAIL) != 0);
  __syncthreads();
}

// Shared-memory layout of a fast block; every array starts on a 16-byte boundary.
struct SmemLayout {
  size_t pose, slot, base8, sph, grp, prm, pairs, flags, cull, qbuf, fkl, hq_n, hq, sdist, total;
};
__host__ __device__ inline size_t a16(size_t x) { return (x + 15) & ~(size_t)15; }
__host__ __device__ inline SmemLayout smem_layout(const PmTablesHdr& h, int cpb, bool want_dist) {
  SmemLayout L;
  size_t o = 0;
  L.pose = o;
  o = a16(o + sizeof(float) * kPoseF * (size_t)cpb * h.n_slots);
  L.slot = o;
  o = a16(o + sizeof(SlotF) * h.n_slots);
  L.base8 = o;
  o = a16(o + sizeof(float) * 8);
  L.sph = o;
  o = a16(o + sizeof(SphereF) * h.n_spheres);
  L.grp = o;
  o = a16(o + sizeof(GroupF) * h.n_groups);
  L.prm = o;
  o = a16(o + sizeof(PrimF) * h.n_prims);
  L.pairs = o;
  o = a16(o + sizeof(int2) * h.n_pairs);
  L.flags = o;
  o = a16(o + sizeof(int) * cpb);
  L.cull = o;
  o = a16(o + sizeof(unsigned) * (size_t)cpb * h.n_groups);
  L.qbuf = o;
  o = a16(o + sizeof(double) * (size_t)cpb * h.q_dim);
  L.fkl = o;
  o = a16(o + 3 * PM_MAX_SLOTS + 3 * sizeof(int));
  L.hq_n = o;
  o = a16(o + 16);
  L.hq = o;
  o = a16(o + (h.n_clouds > 0 ? sizeof(int2) * (size_t)cpb * h.n_spheres : 0));
  L.sdist = o;
  o = a16(o + (want_dist ? sizeof(int) * (size_t)cpb * h.n_spheres : 0));
  L.total = o;
  return L;
}

__device__ Smem carve(unsigned char* p, const PmTablesHdr* T, int cpb) {
  const SmemLayout L = smem_layout(*T, cpb, true);
  Smem sm;
  sm.pose = reinterpret_cast<float*>(p + L.pose);
  sm.slot = reinterpret_cast<SlotF*>(p + L.slot);
  sm.base8 = reinterpret_cast<float*>(p + L.base8);
  sm.sph = reinterpret_cast<SphereF*>(p + L.sph);
  sm.grp = reinterpret_cast<GroupF*>(p + L.grp);
  sm.prm = reinterpret_cast<PrimF*>(p + L.prm);
  sm.pairs = reinterpret_cast<int2*>(p + L.pairs);
  sm.flags = reinterpret_cast<int*>(p + L.flags);
  sm.cull = reinterpret_cast<unsigned*>(p + L.cull);
  sm.qbuf = reinterpret_cast<double*>(p + L.qbuf);
  sm.fkl = p + L.fkl;
  sm.fkn = reinterpret_cast<int*>(p + L.fkl + 3 * PM_MAX_SLOTS);
  sm.hq_n = reinterpret_cast<int*>(p + L.hq_n);
  sm.hq = reinterpret_cast<int2*>(p + L.hq);        // only with a point cloud
  sm.sdist = reinterpret_cast<int*>(p + L.sdist);   // only with distance output (the last array)
  return sm;
}

// The FK slots (FP32, the local transforms' constant parts from the model state) and the fixed base
// pose into shared memory (no barrier).
__device__ void stage_slots(const TView& v, SlotF* __restrict__ slot, float* __restrict__ base8, const double* __restrict__ state) {
  const PmTablesHdr* T = v.T;
  const int tid = threadIdx.x;
  for (int i = tid; i < T->n_slots; i += blockDim.x) {
    const PmSlot& S = v.S[i];
    SlotF f;
    f.parent = S.parent;
    f.mode = S.mode;
    f.qcol = S.qcol;
    f.split = S.split;
    for (int k = 0; k < 3; k++) f.axis[k] = (float)S.axis[k];
    double lt[3];
    if (S.mode == PM_FK_STATE) {
      const double* r = state + (int64_t)PM_STATE_LINK_ROW(S.link) * PM_STATE_STRIDE;
      for (int k = 0; k < 4; k++) f.lq[k] = (float)r[k];
      for (int k = 0; k < 3; k++) lt[k] = r[4 + k];
      f.lid = r[7] != 0.0;
    } else {
      for (int k = 0; k < 4; k++) f.lq[k] = (float)S.oq[k];
      for (int k = 0; k < 3; k++) lt[k] = S.ot[k];
      f.lid = S.origin_identity;
    }
    for (int k = 0; k < 3; k++) f.lt[k] = (float)lt[k];
    f.lt1 = (float)((fabs(lt[0]) + fabs(lt[1]) + fabs(lt[2])) * (1.0 + 1e-6));
    slot[i] = f;
  }
  if (tid < 8) {
    const double* b = state + (int64_t)PM_STATE_BASE_ROW * PM_STATE_STRIDE;
    base8[tid] = tid < 7 ? (float)b[tid] : 0.0f;
  }
}

__device__ void stage_tables(const TView& v, const Smem& sm, const double* __restrict__ state) {
  const PmTablesHdr* T = v.T;
  const int tid = threadIdx.x;
  stage_slots(v, sm.slot, sm.base8, state);
  for (int i = tid; i < T->n_spheres; i += blockDim.x) {
    SphereF s;
    s.x = (float)v.sx[i];
    s.y = (float)v.sy[i];
    s.z = (float)v.sz[i];
    s.r = (float)v.sr[i];
    s.group = v.sgroup[i];
    s.tiny = v.sr[i] < 1e-6;
    s.sn = sqrtf(fmaf(s.x, s.x, fmaf(s.y, s.y, s.z * s.z))) * 1.000002f + 1e-9f;  // rounded up
    sm.sph[i] = s;
  }
  for (int i = tid; i < T->n_groups; i += blockDim.x) {
    const PmGroup& G = v.G[i];
    GroupF g;
    g.rel[0] = (float)G.rel[0];
    g.rel[1] = (float)G.rel[1];
    g.rel[2] = (float)G.rel[2];
    g.radius = (float)G.radius;
    g.slot = G.slot;
    g.begin = G.begin;
    g.count = G.count;
    g.only_self = G.only_self;
    g.tiny = G.radius < 1e-6;
    g.gn = sqrtf(fmaf(g.rel[0], g.rel[0], fmaf(g.rel[1], g.rel[1], g.rel[2] * g.rel[2]))) * 1.000002f + 1e-9f;
    sm.grp[i] = g;
  }
  for (int i = tid; i < T->n_prims; i += blockDim.x) {
    const PmPrim& P = v.P[i];
    PrimF f;
    f.kind = P.kind;
    f.aa = P.axis_aligned;
    f.za = P.z_axis_aligned;
    f.cloud = P.cloud;
    for (int k = 0; k < 3; k++) {
      f.lb[k] = (float)P.lb[k];
      f.ub[k] = (float)P.ub[k];
      f.pos[k] = (float)P.pos[k];
    }
    for (int k = 0; k < 9; k++) f.rot[k] = (float)P.rot[k];
    f.a = (float)P.a;
    f.b = (float)P.b;
    f.c = (float)P.c;
    f.mag = (P.kind == PM_SDF_GROUND || P.kind == PM_SDF_CLOUD)
                ? (float)fabs(P.a)
                : (float)(fabs(P.pos[0]) + fabs(P.pos[1]) + fabs(P.pos[2]) + fabs(P.a) + fabs(P.b) + fabs(P.c));
    sm.prm[i] = f;
  }
  for (int i = tid; i < T->n_pairs; i += blockDim.x) sm.pairs[i] = make_int2(v.pairs[2 * i], v.pairs[2 * i + 1]);
  if (tid == 0) {  // the two-thread FK's slot lists, parents first (the slot order)
    int n[3] = {0, 0, 0};
    for (int i = 0; i < T->n_slots; i++) {
      const int sp = v.S[i].split, l = sp == 0 ? 0 : (sp == 2 ? 1 : 2);
      sm.fkl[l * PM_MAX_SLOTS + n[l]++] = (unsigned char)i;
    }
    for (int l = 0; l < 3; l++) sm.fkn[l] = n[l];
  }
  __syncthreads();
}

// 64 registers a thread, stated as the occupancy target (NT threads x 65536 / (NT x 64) blocks
// per SM): the same budget the compiler picks for NT alone, but its allocation under the explicit
// target measured 4-8 % faster in both modes.
template <int CPB, int NT>
__global__ void __launch_bounds__(NT, 65536 / (NT * 64)) k_fast_valid(const PmTablesHdr* __restrict__ T, const double* __restrict__ state,
                                                    const double* __restrict__ q, int64_t B, uint8_t* __restrict__ out,
                                                    float* __restrict__ dist32, float cutoff, Scratch scr) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  TView v(T);
  Smem sm = carve(smem_raw, T, CPB);
  stage_tables(v, sm, state);
  CfgSource src{q, B, out, scr.bnd};
  const int64_t c0 = (int64_t)blockIdx.x * CPB;
  fast_block<CPB>(v, sm, state, src, c0, (int)(B - c0 < CPB ? B - c0 : CPB), dist32, cutoff, scr, sm.qbuf);
}

// Persistent work-queue kernel over the flattened waypoints of all edges.
// 64 registers a thread as the occupancy target (8 blocks of 128 per SM), as for k_fast_valid:
// 9-15 % faster than the compiler's own choice (72 registers, with spills).
template <int CPB, int NT>
__global__ void __launch_bounds__(NT, 65536 / (NT * 64)) k_fast_edges(const PmTablesHdr* __restrict__ T, const double* __restrict__ state, EdgeSource src,
                                                    unsigned long long* next, Scratch scr) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ long long chunk;
  TView v(T);
  Smem sm = carve(smem_raw, T, CPB);
  stage_tables(v, sm, state);
  const int64_t W = src.E > 0 ? src.off[src.E - 1] + src.n[src.E - 1] : 0;
  for (;;) {
    if (threadIdx.x == 0) chunk = (long long)atomicAdd(next, (unsigned long long)CPB);
    __syncthreads();
    const int64_t c0 = chunk;
    if (c0 >= W) break;
    fast_block<CPB>(v, sm, state, src, c0, (int)(W - c0 < CPB ? W - c0 : CPB), nullptr, 0.f, scr, sm.qbuf);
  }
}

// min(*a, v) for FP32 values of either sign: non-negative floats order like their int bits, negative
// ones in reverse of their unsigned bits.
__device__ __forceinline__ void atomic_min_float(float* a, float v) {
  if (v >= 0.f)
    atomicMin(reinterpret_cast<int*>(a), __float_as_int(v));
  else
    atomicMax(reinterpret_cast<unsigned int*>(a), __float_as_uint(v));
}

// The hard cloud queries of a k_fast_valid launch with distances, two per warp (one per half) over the
// whole queue (no per-block barrier), the next pair's field records read before the current searches
// from query points read one iteration earlier still (so that read is not waited for).
// Same arithmetic as the in-block answer: the distance goes into dist32 by an exact minimum, a certain
// collision clears the configuration, an uncertain one goes to the recheck queue.  A query whose cell
// has no list takes the whole warp's search (warp_nearest32) after the pair's list scans.
// Register budget (64 at 4 blocks of 256 per SM): 32-bit queue indices (the launch allows at most 2^30
// entries), and only the point, reach and cloud held across the search; the fields the result needs are
// read again after it (an L1 hit).  With the whole record held, the kernel spilled and ran 6 % slower.
template <class Src>
__global__ void __launch_bounds__(256, 4) k_hard_queries(const PmTablesHdr* __restrict__ T, const HardQuery* __restrict__ hq,
                                                         float* __restrict__ dist32, Src src, Scratch scr) {
  TView v(T);
  const unsigned FULL = 0xffffffffu;
  const int lane = threadIdx.x & 31, half = lane >> 4, hl = lane & 15;
  const int ns = T->n_spheres;
  const int n = (int)min(*scr.hq_count, (unsigned long long)scr.hq_cap);
  const int nw = (int)((gridDim.x * blockDim.x) >> 5);
  int k = (int)((blockIdx.x * blockDim.x + threadIdx.x) >> 5) * 2;  // the warp's pair: k (half 0), k + 1 (half 1)
  const float4 none = make_float4(__int_as_float(-1), __int_as_float(-1), 0.f, __int_as_float(-1));
  auto point = [&](int i, int& py) {  // the half's query i: its point and packed indices
    py = 0;
    if (i >= n) return make_float4(0.f, 0.f, 0.f, 0.f);
    py = hq[i].b.y;
    return hq[i].a;
  };
  auto record = [&](int i, const float4& qa, int py) {  // field records of query i at point qa
    if (i >= n) return none;
    return field_corner_record(v.C[v.P[(py >> 16) & 0x7fff].cloud], qa.x, qa.y, qa.z, hl);
  };
  int py0, py1;
  const float4 qa0 = point(k + half, py0);
  float4 rec = record(k + half, qa0, py0);
  float4 qa1 = point(k + 2 * nw + half, py1);  // the next query's point, one iteration ahead
  while (k < n) {  // warp-uniform
    const int kn = k + 2 * nw;
    int py2;
    const float4 qa2 = point(kn + 2 * nw + half, py2);  // issued now, used next iteration
    const float4 rec_n = record(kn + half, qa1, py1);
    const int i = k + half;
    const bool have = i < n;  // the same on the half's lanes
    float4 ha = make_float4(0.f, 0.f, 0.f, 0.f);
    int hy = 0;
    if (have) {
      ha = hq[i].a;
      hy = hq[i].b.y;
    }
    const float qx = ha.x, qy = ha.y, qz = ha.z, reach = ha.w;
    const int cloud = have ? v.P[(hy >> 16) & 0x7fff].cloud : 0;  // a half past the end reads cloud 0's constants only
    const FieldStart start = field_corner_candidate(rec, qx, qy, qz, 16);
    const float maxd2 = reach * reach;
    float best = start.nn.d2 < maxd2 ? start.nn.d2 : maxd2;
    int bidx = start.nn.d2 < maxd2 ? start.nn.idx : -1;
    const bool nonfinite = !isfinite(qx) || !isfinite(qy) || !isfinite(qz);
    const int2 rng = have && !nonfinite ? start.rng : make_int2(-1, -1);
    halfwarp_list_nearest32(v.C[cloud], qx, qy, qz, rng, best, bidx);
    // a query without a list: the whole warp's search, one half at a time
    const bool need = have && rng.x < 0;
    for (int hh = 0; hh < 2; hh++) {
      if (__shfl_sync(FULL, need ? 1 : 0, 16 * hh) != 0) {  // warp-uniform
        const float bx = __shfl_sync(FULL, qx, 16 * hh), by = __shfl_sync(FULL, qy, 16 * hh), bz = __shfl_sync(FULL, qz, 16 * hh);
        const float bm = __shfl_sync(FULL, maxd2, 16 * hh), bd = __shfl_sync(FULL, start.nn.d2, 16 * hh);
        const int bi = __shfl_sync(FULL, start.nn.idx, 16 * hh), bc = __shfl_sync(FULL, cloud, 16 * hh);
        const NNResult32 r = warp_nearest32(v.C[bc], bx, by, bz, bm, bd, bi, make_int2(-1, -1));
        if (half == hh) {
          best = r.d2;
          bidx = r.idx;
        }
      }
    }
    if (have && hl == 0) {  // the query's remaining fields, read again after the search
      const int4 hb = hq[i].b;
      const int cfg = hb.x, si = hb.y & 0xffff, prim = (hb.y >> 16) & 0x7fff;
      const bool check = hb.y < 0;
      const float ek = __int_as_float(hb.z);
      const float pa = (float)v.P[prim].a, sr = (float)v.sr[si];
      float g, sd, mag;
      if (bidx < 0) {
        g = reach - pa - sr;
        sd = 3.0e38f;
        mag = fabsf(qx) + fabsf(qy) + fabsf(qz);
      } else {
        const float d = sqrtf(best);
        g = d - pa - sr;
        sd = g;
        mag = fabsf(qx) + fabsf(qy) + fabsf(qz) + d;
      }
      atomic_min_float(dist32 + (int64_t)cfg * ns + si, sd);
      if (check) {
        const float mm = margin32(mag) + ek;
        if (g < -mm) {
          src.fail(cfg);
        } else if (g <= mm) {
          push_item(scr, src, cfg, prim << 1, si, bidx);
        }
      }
    }
    k = kn;
    rec = rec_n;
    qa1 = qa2;
    py1 = py2;
  }
}

// Exact FP64 evaluation of the queued terms, and full plain checks of the configurations (or
// edges) whose terms overflowed the queue.
template <class Src>
__global__ void k_fast_recheck(const PmTablesHdr* __restrict__ T, const double* __restrict__ state, Src src, Scratch scr) {
  TView v(T);
  const unsigned FULL = 0xffffffffu;
  const int lane = threadIdx.x & 31;
  const unsigned int n_items = min(*scr.count, scr.cap);
  double qbuf[PM_MAX_SLOTS + 8];
  // queued terms, one warp per term: lane 0 runs the FP64 FK and the primitive tests, the warp
  // runs the cloud searches
  const int64_t warp = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int64_t n_warps = ((int64_t)gridDim.x * blockDim.x) >> 5;
  for (int64_t i = warp; i < (int64_t)n_items; i += n_warps) {
    const int4 it = scr.items[i];
    if (__shfl_sync(FULL, src.skip(it.x) ? 1 : 0, 0)) continue;
    bool hit = false;
    if (it.y < 0) {  // link-position bound -1 - it.y of a composite constraint, in FP64 (every lane)
      const PmPoseTerm& b = src.bnd.t[-1 - it.y];
      DPose pose[PM_MAX_SLOTS];
      fk64_need_warp(T, state, src.cfg(T, it.x, qbuf), T->base_type == PM_BASE_FIXED, slot_chain(T, b.slot), pose);
      const D3& p = pose[b.slot].t;
      const double x = b.axis == 0 ? p.x : (b.axis == 1 ? p.y : p.z);
      hit = (b.has_lb && x < b.lb) || (b.has_ub && x > b.ub);
    } else if ((it.y & 1) == 0) {  // sphere it.z vs primitive it.y >> 1: gate AND test
      const PmPrim& P = v.P[it.y >> 1];
      const PmGroup& g = v.G[v.sgroup[it.z]];
      // the FP64 FK of the slot's chain of ancestors, by the whole warp (every lane gets the poses)
      DPose pose[PM_MAX_SLOTS];
      fk64_need_warp(T, state, src.cfg(T, it.x, qbuf), T->base_type == PM_BASE_FIXED, slot_chain(T, g.slot), pose);
      const DM3 R = qmat(pose[g.slot].q);
      const D3 gc = add(mv(R, D3{g.rel[0], g.rel[1], g.rel[2]}), pose[g.slot].t);
      const D3 c = add(mv(R, v.rel(it.z)), pose[g.slot].t);
      const double r = v.sr[it.z];
      if (P.kind == PM_SDF_CLOUD) {
        // the sphere's own test first (small reach); its nearest point then settles the gate
        // exactly unless rounding leaves it undecided: min_p |gc - p| <= |gc - p_near|
        const PmGridDev& Gd = v.C[P.cloud];
        int near = -1;
        bool test = !outside_aabb(P, c, r) && !cloud_outside_warp(P, v.C, c, r, &near, it.w);
        if (test && !outside_aabb(P, gc, g.radius)) {
          const D3 d{Gd.px[near] - gc.x, Gd.py[near] - gc.y, Gd.pz[near] - gc.z};
          const double d2n = d.x * d.x + (d.y * d.y + d.z * d.z);
          hit = !(sqrt(d2n) - P.a > g.radius) || !cloud_outside_warp(P, v.C, gc, g.radius, nullptr);
        }
      } else if (lane == 0 && !outside_aabb(P, gc, g.radius) && !prim_outside(P, v.C, gc, g.radius)) {
        hit = !outside_aabb(P, c, r) && !prim_outside(P, v.C, c, r);
      }
    } else {  // sphere pair (it.z, it.w) of self pair it.y >> 1: gate AND test (every lane, same values)
      const int pr = it.y >> 1;
      const PmGroup& g1 = v.G[v.pairs[2 * pr]];
      const PmGroup& g2 = v.G[v.pairs[2 * pr + 1]];
      DPose pose[PM_MAX_SLOTS];
      fk64_need_warp(T, state, src.cfg(T, it.x, qbuf), T->base_type == PM_BASE_FIXED, slot_chain(T, g1.slot) | slot_chain(T, g2.slot),
                     pose);
      const DM3 R1 = qmat(pose[g1.slot].q), R2 = qmat(pose[g2.slot].q);
      const D3 c1 = add(mv(R1, D3{g1.rel[0], g1.rel[1], g1.rel[2]}), pose[g1.slot].t);
      const D3 c2 = add(mv(R2, D3{g2.rel[0], g2.rel[1], g2.rel[2]}), pose[g2.slot].t);
      const double osq = sqn(sub(c1, c2));
      const double ors = g1.radius + g2.radius;
      if (!(osq > ors * ors)) {
        const D3 a = add(mv(R1, v.rel(it.z)), pose[g1.slot].t);
        const D3 bb = add(mv(R2, v.rel(it.w)), pose[g2.slot].t);
        const double rs = v.sr[it.z] + v.sr[it.w];
        hit = sqn(sub(a, bb)) < rs * rs;
      }
    }
    if (__shfl_sync(FULL, hit ? 1 : 0, 0) && lane == 0) src.fail(it.x);
  }
  // configurations (or edges) whose terms overflowed the queue: the plain FP64 check, one thread each
  const int64_t slots = src.n_overflow_slots();
  for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < slots; k += (int64_t)gridDim.x * blockDim.x) {
    if (!scr.overflow[k]) continue;
    src.full_check(v, state, k, qbuf);
    atomicAdd(scr.stats + 2, 1ull);
  }
}

// checkMotion setup: step ratio and number of checked waypoints per edge
// (motion_validator.cpp:17-79, 89-126): n = 0 when the ratio is infinite, else floor(1/r) + 1.
__global__ void k_edge_setup(const double* __restrict__ s1, const double* __restrict__ s2, int64_t E, int dim, int type,
                             const double* __restrict__ width, double resolution, double* __restrict__ sr, int32_t* __restrict__ n,
                             uint8_t* __restrict__ valid) {
  int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (e >= E) return;
  const double* a = s1 + e * dim;
  const double* b = s2 + e * dim;
  double r;
  if (type == 0) {
    double diff_long = 0.0, max_diff = -INFINITY;
    int li = 0;
    for (int i = 0; i < dim; i++) {
      double diff = b[i] - a[i];
      double asd = fabs(diff) * (1.0 / width[i]);
      if (asd > max_diff) {
        max_diff = asd;
        li = i;
        diff_long = diff;
      }
    }
    r = fabs(diff_long) < 1e-6 ? INFINITY : width[li] / fabs(diff_long);
  } else {
    double dist = 0.0;
    for (int i = 0; i < dim; i++) {
      double d = a[i] - b[i];
      dist += d * d;
    }
    r = resolution / sqrt(dist);
  }
  sr[e] = r;
  valid[e] = 1;
  if (r == INFINITY) {
    n[e] = 0;
  } else if (!(r > 0.0) || 1.0 / r > 67108864.0) {  // same bound as the plain kernel
    n[e] = 0;
    valid[e] = 0;
  } else {
    n[e] = (int32_t)(floor(1 / r) + 1);
  }
}

// exclusive scan of n[E] into off[E] with one block (E is at most a few million)
__global__ void k_scan1(const int32_t* __restrict__ n, int64_t E, int64_t* __restrict__ off) {
  __shared__ int64_t part[1024];
  const int tid = threadIdx.x;
  const int64_t per = (E + blockDim.x - 1) / blockDim.x;
  const int64_t b = tid * per, e = min(E, b + per);
  int64_t s = 0;
  for (int64_t i = b; i < e; i++) s += n[i];
  part[tid] = s;
  __syncthreads();
  for (int o = 1; o < (int)blockDim.x; o <<= 1) {
    int64_t t = tid >= o ? part[tid - o] : 0;
    __syncthreads();
    part[tid] += t;
    __syncthreads();
  }
  int64_t run = part[tid] - s;
  for (int64_t i = b; i < e; i++) {
    off[i] = run;
    run += n[i];
  }
}

}  // namespace

namespace pmg {

size_t fast_smem_bytes(const PmTablesHdr& h, int cpb, bool want_dist) { return smem_layout(h, cpb, want_dist).total; }

// Queue records pack a sphere index in 16 bits and a primitive index in 15 (HardQuery.b.y: sphere |
// primitive << 16 | check << 31; the block's queue: configuration << 16 | sphere).  The tables of
// such sizes would not fit in shared memory anyway; the launchers refuse them explicitly.
bool fast_table_sizes_ok(const PmTablesHdr& h) { return h.n_spheres <= 0xffff && h.n_prims <= 0x7fff; }

// Per-device state of this file's kernels: __device__ symbols (the offset table below) exist once
// per device, so each device gets its own upload, and SM counts may differ between devices.
constexpr int kMaxDev = 64;
static std::mutex g_dev_mu;
static bool g_off_done[kMaxDev];
static int g_sm_count[kMaxDev];

static cudaError_t current_device(int* dev) {
  cudaError_t e = cudaGetDevice(dev);
  if (e == cudaSuccess && (*dev < 0 || *dev >= kMaxDev)) e = cudaErrorInvalidDevice;
  return e;
}

// Number of SMs of the current device (cached per device).
cudaError_t sm_count(int* n) {
  int dev = 0;
  cudaError_t e = current_device(&dev);
  if (e != cudaSuccess) return e;
  std::lock_guard<std::mutex> lk(g_dev_mu);
  if (g_sm_count[dev] <= 0) {
    int v = 0;
    if ((e = cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev)) != cudaSuccess) return e;
    g_sm_count[dev] = v > 0 ? v : 1;
  }
  *n = g_sm_count[dev];
  return cudaSuccess;
}

// Uploads the sorted block offsets (c_off, c_off_lb) to the current device, once per device.
cudaError_t upload_offsets() {
  int dev = 0;
  cudaError_t e = current_device(&dev);
  if (e != cudaSuccess) return e;
  std::lock_guard<std::mutex> lk(g_dev_mu);
  if (g_off_done[dev]) return cudaSuccess;
  std::vector<std::pair<float, char4>> v;
  for (int z = -kOffR; z <= kOffR; z++)
    for (int y = -kOffR; y <= kOffR; y++)
      for (int x = -kOffR; x <= kOffR; x++) {
        const float gx = (float)std::max(std::abs(x) - 1, 0), gy = (float)std::max(std::abs(y) - 1, 0), gz = (float)std::max(std::abs(z) - 1, 0);
        // exact-below lower bound: rounded down by one part in 1e6
        const float lb = std::sqrt(gx * gx + gy * gy + gz * gz) * (1.0f - 1e-6f);
        v.push_back({lb, make_char4((char)x, (char)y, (char)z, 0)});
      }
  std::stable_sort(v.begin(), v.end(), [](const std::pair<float, char4>& a, const std::pair<float, char4>& b) {
    if (a.first != b.first) return a.first < b.first;
    const int da = a.second.x * a.second.x + a.second.y * a.second.y + a.second.z * a.second.z;
    const int db = b.second.x * b.second.x + b.second.y * b.second.y + b.second.z * b.second.z;
    return da < db;
  });
  std::vector<char4> off(v.size());
  std::vector<float> lb(v.size());
  for (size_t i = 0; i < v.size(); i++) {
    off[i] = v[i].second;
    lb[i] = v[i].first;
  }
  e = cudaMemcpyToSymbol(c_off, off.data(), off.size() * sizeof(char4));
  if (e == cudaSuccess) e = cudaMemcpyToSymbol(c_off_lb, lb.data(), lb.size() * sizeof(float));
  if (e == cudaSuccess) g_off_done[dev] = true;
  return e;
}

// The offset table on the device and the kernel's dynamic shared-memory limit raised to sm bytes;
// both once per device (the attribute again only for a larger size), so small calls pay for neither.
template <class K>
static cudaError_t prep(K kern, size_t sm) {
  cudaError_t e = upload_offsets();
  if (e != cudaSuccess) return e;
  int dev = 0;
  if ((e = current_device(&dev)) != cudaSuccess) return e;
  static std::mutex mu;
  static std::map<std::pair<const void*, int>, size_t> raised;
  std::lock_guard<std::mutex> lk(mu);
  size_t& have = raised[{reinterpret_cast<const void*>(kern), dev}];
  if (have >= sm) return cudaSuccess;
  e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
  if (e == cudaSuccess) have = sm;
  return e;
}

// Blocks of the recheck kernel: one 4-warp block per 32 configurations (or 8 edges), at most 4 per
// SM; its loops stride over the grid, so a small batch launches few blocks.
static unsigned recheck_grid(int64_t units, int per_block, int n_sm) {
  const int64_t want = (units + per_block - 1) / per_block;
  return (unsigned)std::max<int64_t>(1, std::min<int64_t>(want, (int64_t)n_sm * 4));
}

// count, overflow and stats must be zeroed by the caller
cudaError_t launch_fast_valid(const PmTablesHdr* T, const PmTablesHdr& h, const double* state, const double* q, int64_t B,
                              uint8_t* out, float* dist32, float cutoff, int4* items, unsigned int* count, unsigned int cap,
                              uint8_t* overflow, unsigned long long* stats, int cpb, int nt, cudaStream_t s, void* hq,
                              unsigned long long* hq_count, unsigned int hq_cap, const FastTuning& tune, PmLinkBounds bnd) {
  if (B <= 0) return cudaSuccess;
  if (!fast_table_sizes_ok(h)) return cudaErrorInvalidConfiguration;
  // (hard-query entries hold 32-bit configuration indices)
  // k_hard_queries indexes its queue in 32 bits: at most 2^30 entries
  const bool split = dist32 != nullptr && hq != nullptr && hq_count != nullptr && hq_cap > 0 && hq_cap <= (1u << 30) &&
                     h.n_clouds > 0 && B <= 0x7fffffffLL;
  Scratch scr{items, count, cap, overflow, stats, split ? static_cast<HardQuery*>(hq) : nullptr, split ? hq_count : nullptr,
              split ? hq_cap : 0u, tune.sphere_tile_log2, bnd};
  size_t sm = fast_smem_bytes(h, cpb, dist32 != nullptr);
  if (sm > 200 * 1024) return cudaErrorInvalidConfiguration;
  unsigned grid = (unsigned)((B + cpb - 1) / cpb);
  cudaError_t e;
  prof_begin("k_fast_valid", s);
#define PM_FAST_CASE(C, N)                                                                      \
  if (cpb == C && nt == N) {                                                                     \
    if ((e = prep(k_fast_valid<C, N>, sm)) != cudaSuccess) return e;                             \
    k_fast_valid<C, N><<<grid, N, sm, s>>>(T, state, q, B, out, dist32, cutoff, scr);            \
    launched = true;                                                                             \
  }
  bool launched = false;
  PM_FAST_CASE(16, 128)
  PM_FAST_CASE(32, 128)
  PM_FAST_CASE(16, 256)
  PM_FAST_CASE(32, 256)
  PM_FAST_CASE(64, 256)
  PM_FAST_CASE(32, 512)
  PM_FAST_CASE(64, 512)
  PM_FAST_CASE(128, 512)
#undef PM_FAST_CASE
  if (!launched) return cudaErrorInvalidValue;
  if ((e = cudaGetLastError()) != cudaSuccess) return e;
  prof_end("k_fast_valid", s);
  CfgSource src{q, B, out, bnd};
  int n_sm = 0;
  if ((e = sm_count(&n_sm)) != cudaSuccess) return e;
  if (split) {
    prof_begin("k_hard_queries", s);
    const int bps = tune.hq_blocks_per_sm >= 1 && tune.hq_blocks_per_sm <= 8 ? tune.hq_blocks_per_sm : 4;
    k_hard_queries<CfgSource><<<n_sm * bps, 256, 0, s>>>(T, scr.hq, dist32, src, scr);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    prof_end("k_hard_queries", s);
  }
  prof_begin("k_fast_recheck", s);
  k_fast_recheck<CfgSource><<<recheck_grid(B, 32, n_sm), 128, 0, s>>>(T, state, src, scr);
  prof_end("k_fast_recheck", s);
  return cudaGetLastError();
}

// work: sr (E doubles), n (E int32), off (E int64), next (1 ull), all device; count/overflow(E)/
// stats/next zeroed by the caller.  out receives the edge booleans.
cudaError_t launch_fast_edges(const PmTablesHdr* T, const PmTablesHdr& h, const double* state, const double* s1, const double* s2,
                              int64_t E, int type, const double* width, double resolution, const int16_t* seq, double* sr, int32_t* n,
                              int64_t* off, unsigned long long* next, uint8_t* out, int4* items, unsigned int* count,
                              unsigned int cap, uint8_t* overflow, unsigned long long* stats, int cpb, int nt, int n_sm, cudaStream_t s,
                              PmLinkBounds bnd) {
  if (E <= 0) return cudaSuccess;
  if (!fast_table_sizes_ok(h)) return cudaErrorInvalidConfiguration;
  Scratch scr{items, count, cap, overflow, stats};
  k_edge_setup<<<(unsigned)((E + 127) / 128), 128, 0, s>>>(s1, s2, E, h.q_dim, type, width, resolution, sr, n, out);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  k_scan1<<<1, 1024, 0, s>>>(n, E, off);
  if ((e = cudaGetLastError()) != cudaSuccess) return e;
  EdgeSource src{s1, s2, off, n, sr, seq, E, out, bnd};
  size_t sm = fast_smem_bytes(h, cpb, false);
  if (sm > 200 * 1024) return cudaErrorInvalidConfiguration;
  bool launched = false;
  // persistent blocks, at most 4 per edge (a few chunks of waypoints each): a small call stages the
  // tables in few blocks
#define PM_EDGE_CASE(C, N)                                                                                               \
  if (cpb == C && nt == N) {                                                                                              \
    int per_sm = 0;                                                                                                      \
    if ((e = prep(k_fast_edges<C, N>, sm)) != cudaSuccess) return e;                                                      \
    if ((e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_fast_edges<C, N>, N, sm)) != cudaSuccess) return e; \
    const unsigned grid = (unsigned)std::min<int64_t>((int64_t)n_sm * (per_sm > 0 ? per_sm : 1), std::max<int64_t>(1, 4 * E)); \
    prof_begin("k_fast_edges", s);                                                                                        \
    k_fast_edges<C, N><<<grid, N, sm, s>>>(T, state, src, next, scr);                                                     \
    prof_end("k_fast_edges", s);                                                                                          \
    launched = true;                                                                                                     \
  }
  PM_EDGE_CASE(16, 128)
  PM_EDGE_CASE(32, 128)
  PM_EDGE_CASE(32, 256)
  PM_EDGE_CASE(64, 256)
#undef PM_EDGE_CASE
  if (!launched) return cudaErrorInvalidValue;
  if ((e = cudaGetLastError()) != cudaSuccess) return e;
  prof_begin("k_fast_recheck_edges", s);
  k_fast_recheck<EdgeSource><<<recheck_grid(E, 8, n_sm), 128, 0, s>>>(T, state, src, scr);
  prof_end("k_fast_recheck_edges", s);
  return cudaGetLastError();
}

}  // namespace pmg
