// Differentiable costs in FP32 with a hand-written reverse-mode adjoint: batched collision-aware
// IK (cost, gradient, and whole gradient-descent runs in one launch) and trajectory smoothing
// with the collision hinge (FK recomputed per waypoint in the backward pass, nothing stored).
//
// A unit of GW lanes per IK problem (16: two problems per warp) or per trajectory waypoint (a warp).
// Per evaluation:
//   1. FK: lanes build the slots' local transforms (sincosf); with a slot per lane, pointer jumping
//      over the slot tree composes the world poses in ceil(log2(depth + 1)) steps (else the unit's
//      first lane composes them parents-first); lanes turn the world quaternions into rotation
//      matrices;
//   2. spheres: per slot, the primitives the slot's bounding sphere leaves within the threshold;
//      then each lane takes spheres (ordered by slot) and computes d_s = min over those primitives
//      of evaluate(c) - r (the SphereCollisionCst ext-row value, primitive_sphere_collision.cpp:
//      256-322), skipping primitives whose bounding-sphere lower bound is already past the
//      threshold, with the analytic SDF gradient of the argmin primitive;
//   3. adjoint: the cost's gradient with respect to each sphere centre is a force at the centre;
//      forces and moments are summed per slot, then over each subtree (a prefix sum over the lanes
//      in DFS order, moments about the world origin; else children first on one lane), and a
//      revolute joint's derivative is its world axis dotted with the moment about its origin
//      (prismatic: with the force).  This is the transpose of the attached-point Jacobian of
//      algorithm.cpp:346-380 applied to every sphere at once, in O(slots + spheres).
// The pose term ||p - p*||^2 + w_rot ||log(R*^T R)||^2 adds a force 2 w_pos (p - p*) at the pose
// link origin and a pure moment 2 w_rot R* phi (phi the rotation vector of R*^T R; phi is an
// eigenvector of the inverse left Jacobian, so the chain rule reduces to that moment).
#include <algorithm>
#include <cmath>

#include "pm_grad.cuh"
#include "pm_grid.cuh"
#include "pm_launch.h"
#include "pm_math.cuh"

using namespace pmd;

namespace {

constexpr int kNW = 8;  // warps per block

struct GSlot {
  int parent, mode, qcol, lid;
  float axis[3];
  float lq[4];  // REV: joint origin rotation; STATE: the fixed local rotation
  float lt[3];  // joint origin / fixed local translation
  int send;     // one past the last slot of this slot's subtree (subtrees are contiguous in slot order)
};
struct alignas(16) GSph {  // 32 bytes: one 16-byte and one 8-byte shared-memory load per sphere
  float x, y, z, r;
  int slot, active;  // active: takes part in the ext cost (its group is not self-only)
  int pad0, pad1;
};
struct alignas(16) GPrim {  // pos and bound in one 16-byte load
  int kind, aa, cloud, pad;
  float pos[3], bound;  // bound: radius of a sphere around pos containing the primitive (<0: no cull)
  float rot[9];
  float a, b, c, pad2;
};
constexpr int kSlotF = 33;  // floats of per-unit work per slot (odd: lanes on different slots use different banks)

// Passed by value as a kernel argument: its fields are read from parameter space wherever they are used,
// so the header values copied here (n_ctrl, base_type, off_clouds: set by the launcher from the host
// copy of the header) hold no registers across the cost (the IK kernel spills at its 64 registers).
struct Layout {
  int n_slots, n_sph, n_prims, qd, qpad, n_ctrl, base_type;
  int64_t off_clouds;
  size_t off_slots, off_sph, off_sbeg, off_prims, off_sbnd, off_warp, warp_floats, total;
};

__host__ __device__ inline size_t al16(size_t x) { return (x + 15) & ~(size_t)15; }

// groups: units in flight per block (kNW warps times the units per warp)
__host__ __device__ inline Layout make_layout(int n_slots, int n_sph, int n_prims, int qd, int groups = kNW) {
  Layout L;
  L.n_slots = n_slots;
  L.n_sph = n_sph;
  L.n_prims = n_prims;
  L.qd = qd;
  L.qpad = (qd + 3) & ~3;
  size_t o = 0;
  L.off_slots = o;
  o = al16(o + sizeof(GSlot) * n_slots);
  L.off_sph = o;
  o = al16(o + sizeof(GSph) * n_sph);
  L.off_sbeg = o;
  o = al16(o + sizeof(int) * (n_slots + 1));
  L.off_prims = o;
  o = al16(o + sizeof(GPrim) * n_prims);
  L.off_sbnd = o;
  o = al16(o + sizeof(float4) * n_slots);
  L.off_warp = o;
  // per warp: q, grad, target/pose wrench scratch (16), slot work, sphere adjoints (6 each)
  L.warp_floats = (size_t)2 * L.qpad + 16 + (size_t)kSlotF * n_slots + (size_t)6 * n_sph;
  L.warp_floats = (L.warp_floats + 3) & ~(size_t)3;
  L.total = o + sizeof(float) * L.warp_floats * groups;
  return L;
}

struct Tab {
  const GSlot* slot;
  const GSph* sph;
  const int* sbeg;
  const GPrim* prim;
  const float4* sbnd;  // per slot: a sphere in the slot frame containing its active spheres (w < 0: none)
  const PmGridDev* clouds;
  int n_slots, n_sph, n_prims, qd, n_ctrl, base_type;
};
// the fixed base pose ([0..3] quaternion, [4..6] translation) and the subtree-range flag of the block
__shared__ float g_base_pose[8];
__shared__ int g_tree_bad;

// Stage the constraint tables into shared memory in FP32 (once per block).
__device__ void stage(const PmTablesHdr* T, const double* state, const Layout& L, char* smem, Tab& t) {
  GSlot* sl = (GSlot*)(smem + L.off_slots);
  GSph* sp = (GSph*)(smem + L.off_sph);
  int* sb = (int*)(smem + L.off_sbeg);
  GPrim* pr = (GPrim*)(smem + L.off_prims);
  const PmSlot* S = pm_at<PmSlot>(T, T->off_slots);
  const PmGroup* G = pm_at<PmGroup>(T, T->off_groups);
  const double* sx = pm_at<double>(T, T->off_sx);
  const double* sy = pm_at<double>(T, T->off_sy);
  const double* sz = pm_at<double>(T, T->off_sz);
  const double* sr = pm_at<double>(T, T->off_sr);
  const int32_t* sg = pm_at<int32_t>(T, T->off_sgroup);
  const PmPrim* P = pm_at<PmPrim>(T, T->off_prims);
  for (int i = threadIdx.x; i < L.n_slots; i += blockDim.x) {
    const PmSlot& s = S[i];
    GSlot g;
    g.parent = s.parent;
    g.mode = s.mode;
    g.qcol = s.qcol;
    for (int k = 0; k < 3; k++) g.axis[k] = (float)s.axis[k];
    if (s.mode == PM_FK_STATE) {
      const double* r = state + (int64_t)PM_STATE_LINK_ROW(s.link) * PM_STATE_STRIDE;
      for (int k = 0; k < 4; k++) g.lq[k] = (float)r[k];
      for (int k = 0; k < 3; k++) g.lt[k] = (float)r[4 + k];
      g.lid = r[7] != 0.0;
    } else {
      for (int k = 0; k < 4; k++) g.lq[k] = (float)s.oq[k];
      for (int k = 0; k < 3; k++) g.lt[k] = (float)s.ot[k];
      g.lid = s.origin_identity;
    }
    sl[i] = g;
  }
  if (threadIdx.x == 0) {  // spheres ordered by slot (stable): counting sort
    for (int i = 0; i <= L.n_slots; i++) sb[i] = 0;
    for (int k = 0; k < L.n_sph; k++) sb[G[sg[k]].slot + 1]++;
    for (int i = 0; i < L.n_slots; i++) sb[i + 1] += sb[i];
  }
  __syncthreads();
  for (int k = threadIdx.x; k < L.n_sph; k += blockDim.x) {
    const int slot = G[sg[k]].slot;
    int pos = sb[slot];
    for (int j = 0; j < k; j++) pos += G[sg[j]].slot == slot;
    sp[pos] = GSph{(float)sx[k], (float)sy[k], (float)sz[k], (float)sr[k], slot, !G[sg[k]].only_self};
  }
  for (int i = threadIdx.x; i < L.n_prims; i += blockDim.x) {
    const PmPrim& p = P[i];
    GPrim g;
    g.kind = p.kind;
    g.aa = p.kind == PM_SDF_BOX ? p.axis_aligned : 0;
    g.cloud = p.cloud;
    g.pad = 0;
    for (int k = 0; k < 3; k++) g.pos[k] = (float)p.pos[k];
    for (int k = 0; k < 9; k++) g.rot[k] = (float)p.rot[k];
    g.a = (float)p.a;
    g.b = (float)p.b;
    g.c = (float)p.c;
    g.pad2 = 0.f;
    switch (p.kind) {
      case PM_SDF_BOX: g.bound = (float)sqrt(p.a * p.a + p.b * p.b + p.c * p.c) * (1.f + 1e-6f); break;
      case PM_SDF_CYLINDER: g.bound = (float)sqrt(p.a * p.a + p.c * p.c) * (1.f + 1e-6f); break;
      case PM_SDF_SPHERE: g.bound = (float)p.a * (1.f + 1e-6f); break;
      default: g.bound = -1.f;
    }
    pr[i] = g;
  }
  __syncthreads();
  // subtree ranges: slot i's subtree is [i, send) when the slots are in DFS preorder (checked)
  if (threadIdx.x == 0) g_tree_bad = 0;
  __syncthreads();
  for (int i = threadIdx.x; i < L.n_slots; i += blockDim.x) {
    int e = i + 1;
    while (e < L.n_slots) {  // the first later slot outside i's subtree
      int a = sl[e].parent;
      while (a > i) a = sl[a].parent;
      if (a != i) break;
      e++;
    }
    for (int j = e; j < L.n_slots; j++) {  // no later slot may fall back into the subtree
      int a = sl[j].parent;
      while (a > i) a = sl[a].parent;
      if (a == i) g_tree_bad = 1;
    }
    sl[i].send = e;
  }
  __syncthreads();
  // per slot: centre = mean of its active spheres' centres, radius = the largest |c_j - centre| + r_j,
  // widened by 1e-5 relative + 1 um so that it also holds the FP32 sphere centres of the cost
  float4* bs = (float4*)(smem + L.off_sbnd);
  for (int i = threadIdx.x; i < L.n_slots; i += blockDim.x) {
    float cx = 0.f, cy = 0.f, cz = 0.f;
    int n = 0;
    for (int k = sb[i]; k < sb[i + 1]; k++)
      if (sp[k].active) {
        cx += sp[k].x;
        cy += sp[k].y;
        cz += sp[k].z;
        n++;
      }
    float R = -1.f;
    if (n > 0) {
      cx /= (float)n;
      cy /= (float)n;
      cz /= (float)n;
      R = 0.f;
      for (int k = sb[i]; k < sb[i + 1]; k++)
        if (sp[k].active) {
          const float dx = sp[k].x - cx, dy = sp[k].y - cy, dz = sp[k].z - cz;
          R = fmaxf(R, sqrtf(fmaf(dx, dx, fmaf(dy, dy, dz * dz))) + sp[k].r);
        }
      R = R * (1.f + 1e-5f) + 1e-6f;
    }
    bs[i] = make_float4(cx, cy, cz, R);
  }
  t.slot = sl;
  t.sph = sp;
  t.sbeg = sb;
  t.prim = pr;
  t.sbnd = bs;
  t.clouds = pm_at<PmGridDev>(T, L.off_clouds);
  t.n_slots = L.n_slots;
  t.n_sph = L.n_sph;
  t.n_prims = L.n_prims;
  t.qd = L.qd;
  t.n_ctrl = L.n_ctrl;
  t.base_type = L.base_type;
  const double* b = state + (int64_t)PM_STATE_BASE_ROW * PM_STATE_STRIDE;
  if (threadIdx.x < 7) g_base_pose[threadIdx.x] = (float)b[threadIdx.x];
  __syncthreads();
}

// Per-warp scratch views.
struct WS {
  float* q;     // qpad
  float* g;     // qpad
  float* misc;  // 16: pose wrench (6)
  float* sw;    // slots x kSlotF: [0..3] local q, [4..6] local t, [7] local-identity flag,
                //                 [8..11] world q, [12..14] world t, [16..24] R, [25..27] F, [28..30] moment
  float* sadj;  // spheres x 6: force and moment about the slot origin
};
__device__ __forceinline__ WS warp_ws(const Layout& L, char* smem, int w) {
  float* base = (float*)(smem + L.off_warp) + (size_t)w * L.warp_floats;
  WS s;
  s.q = base;
  s.g = base + L.qpad;
  s.misc = base + 2 * L.qpad;
  s.sw = s.misc + 16;
  s.sadj = s.sw + (size_t)kSlotF * L.n_slots;
  return s;
}

// Sum over a unit's GW lanes (a whole warp, or each aligned GW-lane part of it: the xor offsets
// stay inside).
template <int GW = 32>
__device__ __forceinline__ float warp_sum(float v) {
  for (int o = GW / 2; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

__device__ __forceinline__ void cross3(const float a[3], const float b[3], float o[3]) {
  o[0] = fmaf(a[1], b[2], -a[2] * b[1]);
  o[1] = fmaf(a[2], b[0], -a[0] * b[2]);
  o[2] = fmaf(a[0], b[1], -a[1] * b[0]);
}

// FK of the unit's configuration ws.q into ws.sw (GW lanes per unit; the units of a warp run it
// in step).
template <int GW = 32>
__device__ void warp_fk(const Tab& t, const WS& ws, int lane) {
  for (int i = lane; i < t.n_slots; i += GW) {
    const GSlot& s = t.slot[i];
    float* w = ws.sw + (size_t)i * kSlotF;
    if (s.parent < 0) continue;
    if (s.mode == PM_FK_STATE) {
      for (int k = 0; k < 4; k++) w[k] = s.lq[k];
      for (int k = 0; k < 3; k++) w[4 + k] = s.lt[k];
      w[7] = (float)s.lid;
      continue;
    }
    const float th = ws.q[s.qcol];
    if (s.mode == PM_FK_PRIS) {
      w[0] = w[1] = w[2] = 0.f;
      w[3] = 1.f;
      for (int k = 0; k < 3; k++) w[4 + k] = fmaf(s.axis[k], th, s.lt[k]);
      w[7] = 1.f;
      continue;
    }
    float sn, cs;
    sincosf(th * 0.5f, &sn, &cs);
    FQ jq{sn * s.axis[0], sn * s.axis[1], sn * s.axis[2], cs};
    FQ lq = s.lid ? jq : fqmul(FQ{s.lq[0], s.lq[1], s.lq[2], s.lq[3]}, jq);
    w[0] = lq.x;
    w[1] = lq.y;
    w[2] = lq.z;
    w[3] = lq.w;
    for (int k = 0; k < 3; k++) w[4 + k] = s.lt[k];
    w[7] = 0.f;
  }
  __syncwarp();
  // world poses, parents first: the base pose at the root, then T_i = T_parent(i) o local_i
  auto base_pose = [&](FQ& bq, float bt[3]) {
    bq = FQ{g_base_pose[0], g_base_pose[1], g_base_pose[2], g_base_pose[3]};
    bt[0] = g_base_pose[4];
    bt[1] = g_base_pose[5];
    bt[2] = g_base_pose[6];
    if (t.base_type == PM_BASE_PLANAR) {
      const float* qb = ws.q + t.n_ctrl;
      float sn, cs;
      sincosf(qb[2] * 0.5f, &sn, &cs);
      bq = FQ{0.f, 0.f, sn, cs};
      bt[0] = qb[0];
      bt[1] = qb[1];
      bt[2] = 0.f;
    } else if (t.base_type == PM_BASE_FLOATING) {
      const float* qb = ws.q + t.n_ctrl;
      float sr, cr, sp, cp, sy, cy;
      sincosf(qb[3] * 0.5f, &sr, &cr);
      sincosf(qb[4] * 0.5f, &sp, &cp);
      sincosf(qb[5] * 0.5f, &sy, &cy);
      bq = FQ{sr * cp * cy - cr * sp * sy, cr * sp * cy + sr * cp * sy, cr * cp * sy - sr * sp * cy, cr * cp * cy + sr * sp * sy};
      bt[0] = qb[0];
      bt[1] = qb[1];
      bt[2] = qb[2];
    }
  };
  if (t.n_slots <= GW) {
    // one slot per lane, pointer jumping over the slot tree: each step composes the transform
    // accumulated so far with that of the current ancestor and jumps to the ancestor's ancestor,
    // so depth d takes ceil(log2(d + 1)) steps (a chain of 8 slots: 3) instead of d serial ones
    const unsigned FULL = 0xffffffffu;
    const int i = lane;
    const bool own = i < t.n_slots;
    FQ q{0.f, 0.f, 0.f, 1.f};
    float tr[3] = {0.f, 0.f, 0.f};
    int anc = -1;
    if (own) {
      const float* w = ws.sw + (size_t)i * kSlotF;
      anc = t.slot[i].parent;
      if (anc < 0) {
        base_pose(q, tr);
      } else {
        q = w[7] != 0.f ? FQ{0.f, 0.f, 0.f, 1.f} : FQ{w[0], w[1], w[2], w[3]};  // flagged identity, as the serial path
        tr[0] = w[4];
        tr[1] = w[5];
        tr[2] = w[6];
      }
    }
    while (__any_sync(FULL, anc >= 0)) {  // warp-uniform
      const int src = anc >= 0 ? anc : i;
      const FQ aq{__shfl_sync(FULL, q.x, src, GW), __shfl_sync(FULL, q.y, src, GW), __shfl_sync(FULL, q.z, src, GW),
                  __shfl_sync(FULL, q.w, src, GW)};
      const float at[3] = {__shfl_sync(FULL, tr[0], src, GW), __shfl_sync(FULL, tr[1], src, GW), __shfl_sync(FULL, tr[2], src, GW)};
      const int aa = __shfl_sync(FULL, anc, src, GW);
      if (anc >= 0) {
        float r[3];
        fqrot(aq, tr, r);
        tr[0] = at[0] + r[0];
        tr[1] = at[1] + r[1];
        tr[2] = at[2] + r[2];
        q = fqmul(aq, q);
        anc = aa;
      }
    }
    if (own) {
      float* w = ws.sw + (size_t)i * kSlotF;
      w[8] = q.x;
      w[9] = q.y;
      w[10] = q.z;
      w[11] = q.w;
      w[12] = tr[0];
      w[13] = tr[1];
      w[14] = tr[2];
    }
  } else if (lane == 0) {
    for (int i = 0; i < t.n_slots; i++) {
      const GSlot& s = t.slot[i];
      float* w = ws.sw + (size_t)i * kSlotF;
      if (s.parent < 0) {
        FQ bq;
        float bt[3];
        base_pose(bq, bt);
        w[8] = bq.x;
        w[9] = bq.y;
        w[10] = bq.z;
        w[11] = bq.w;
        for (int k = 0; k < 3; k++) w[12 + k] = bt[k];
        continue;
      }
      const float* pw = ws.sw + (size_t)s.parent * kSlotF;
      const FQ pq{pw[8], pw[9], pw[10], pw[11]};
      float r[3];
      fqrot(pq, w + 4, r);
      for (int k = 0; k < 3; k++) w[12 + k] = pw[12 + k] + r[k];
      const FQ cq = w[7] != 0.f ? pq : fqmul(pq, FQ{w[0], w[1], w[2], w[3]});
      w[8] = cq.x;
      w[9] = cq.y;
      w[10] = cq.z;
      w[11] = cq.w;
    }
  }
  __syncwarp();
  for (int i = lane; i < t.n_slots; i += GW) {
    float* w = ws.sw + (size_t)i * kSlotF;
    fqmat(FQ{w[8], w[9], w[10], w[11]}, w + 16);
  }
  __syncwarp();
}

// evaluate() of a box / cylinder / sphere / ground primitive at c (the reference's signed
// distances, primitive_sdf.hpp) and its analytic gradient.  Inside a box the gradient is the
// normal of the face of largest s_k; inside a cylinder, of the larger of the radial and axial
// terms (the subgradient the value follows).
__device__ __forceinline__ float prim_value_grad(const GPrim& P, const float c[3], float g[3]) {
  const float dx = c[0] - P.pos[0], dy = c[1] - P.pos[1], dz = c[2] - P.pos[2];
  g[0] = g[1] = g[2] = 0.f;
  if (P.kind == PM_SDF_SPHERE) {
    const float n = sqrtf(fmaf(dx, dx, fmaf(dy, dy, dz * dz)));
    if (n > 0.f) {
      const float inv = 1.f / n;
      g[0] = dx * inv;
      g[1] = dy * inv;
      g[2] = dz * inv;
    }
    return n - P.a;
  }
  if (P.kind == PM_SDF_GROUND) {
    g[2] = 1.f;
    return c[2] + P.a;
  }
  const float* R = P.rot;  // world-from-primitive, row-major
  float l[3];
  if (P.aa) {
    l[0] = dx;
    l[1] = dy;
    l[2] = dz;
  } else {
    l[0] = fmaf(dx, R[0], fmaf(dy, R[3], dz * R[6]));
    l[1] = fmaf(dx, R[1], fmaf(dy, R[4], dz * R[7]));
    l[2] = fmaf(dx, R[2], fmaf(dy, R[5], dz * R[8]));
  }
  float gl[3] = {0.f, 0.f, 0.f};
  float val;
  if (P.kind == PM_SDF_BOX) {
    const float s0 = fabsf(l[0]) - P.a, s1 = fabsf(l[1]) - P.b, s2 = fabsf(l[2]) - P.c;
    const float m0 = fmaxf(s0, 0.f), m1 = fmaxf(s1, 0.f), m2 = fmaxf(s2, 0.f);
    const float out = sqrtf(fmaf(m0, m0, fmaf(m1, m1, m2 * m2)));
    if (out > 0.f) {
      const float inv = 1.f / out;
      gl[0] = copysignf(m0 * inv, l[0]);
      gl[1] = copysignf(m1 * inv, l[1]);
      gl[2] = copysignf(m2 * inv, l[2]);
      val = out;
    } else if (s0 >= s1 && s0 >= s2) {
      gl[0] = copysignf(1.f, l[0]);
      val = s0;
    } else if (s1 >= s2) {
      gl[1] = copysignf(1.f, l[1]);
      val = s1;
    } else {
      gl[2] = copysignf(1.f, l[2]);
      val = s2;
    }
  } else {  // cylinder: a = radius, c = half height, axis = local z
    const float rho = sqrtf(fmaf(l[0], l[0], l[1] * l[1]));
    const float rs = rho - P.a, zs = fabsf(l[2]) - P.c;
    const float inv_rho = rho > 0.f ? 1.f / rho : 0.f;
    const float ux = rho > 0.f ? l[0] * inv_rho : 1.f, uy = l[1] * inv_rho;
    const float ma = fmaxf(rs, 0.f), mb = fmaxf(zs, 0.f);
    const float out = sqrtf(fmaf(ma, ma, mb * mb));
    if (out > 0.f) {
      const float inv = 1.f / out;
      gl[0] = ux * ma * inv;
      gl[1] = uy * ma * inv;
      gl[2] = copysignf(mb * inv, l[2]);
      val = out;
    } else if (rs >= zs) {
      gl[0] = ux;
      gl[1] = uy;
      val = rs;
    } else {
      gl[2] = copysignf(1.f, l[2]);
      val = zs;
    }
  }
  if (P.aa) {
    g[0] = gl[0];
    g[1] = gl[1];
    g[2] = gl[2];
  } else {
    g[0] = fmaf(R[0], gl[0], fmaf(R[1], gl[1], R[2] * gl[2]));
    g[1] = fmaf(R[3], gl[0], fmaf(R[4], gl[1], R[5] * gl[2]));
    g[2] = fmaf(R[6], gl[0], fmaf(R[7], gl[1], R[8] * gl[2]));
  }
  return val;
}

// d_s of one sphere centre: min over primitives (lower bound below thr) of evaluate - r, with the
// gradient of the argmin primitive.  +inf (zero gradient) when every primitive is past thr.
// mask: the primitives its slot's bounding sphere leaves in reach (bit j: primitive j; all primitives
// beyond 32 are tested).
__device__ __forceinline__ float sphere_min_dist(const Tab& t, const float c[3], float r, float thr, float grad[3], unsigned mask) {
  float best = INFINITY;
  grad[0] = grad[1] = grad[2] = 0.f;
  for (int j = t.n_prims <= 32 ? (mask ? __ffs(mask) - 1 : t.n_prims) : 0; j < t.n_prims;) {
    const GPrim& P = t.prim[j];
    const int jn = j + 1;
    // the next primitive: the next set bit of the mask (or the next index beyond 32 primitives)
    j = t.n_prims <= 32 ? ((mask &= mask - 1) ? __ffs(mask) - 1 : t.n_prims) : jn;
    if (P.bound >= 0.f) {
      const float dx = c[0] - P.pos[0], dy = c[1] - P.pos[1], dz = c[2] - P.pos[2];
      const float lb = sqrtf(fmaf(dx, dx, fmaf(dy, dy, dz * dz))) - P.bound - r;
      if (lb >= thr || lb >= best) continue;
    }
    float g[3];
    float v;
    if (P.kind == PM_SDF_CLOUD) {  // nearest point closer than the current best / threshold
      const PmGridDev& G = t.clouds[P.cloud];
      const float reach = fminf(thr, best) + r + P.a;
      if (!(reach > 0.f)) continue;
      const FieldLB fb = grid_field32(G, c[0], c[1], c[2]);
      if (fb.lb >= reach) continue;
      // the field cell's nearest point bounds the walk; the walk reports only strictly closer points
      const float d2_0 = fb.idx >= 0 ? point_d2_32(G, fb.idx, c[0], c[1], c[2]) : INFINITY;
      NNResult32 nn = grid_nearest32(G, c[0], c[1], c[2], fminf(reach * reach, d2_0));
      if (nn.idx < 0 && d2_0 < reach * reach) nn = NNResult32{d2_0, fb.idx};
      if (nn.idx < 0) continue;
      const float4 p = __ldg(G.p32 + nn.idx);
      const float ex = c[0] - p.x, ey = c[1] - p.y, ez = c[2] - p.z;
      const float n = sqrtf(nn.d2);
      g[0] = g[1] = g[2] = 0.f;
      if (n > 0.f) {
        const float inv = 1.f / n;
        g[0] = ex * inv;
        g[1] = ey * inv;
        g[2] = ez * inv;
      }
      v = n - P.a;
    } else {
      v = prim_value_grad(P, c, g);
    }
    v -= r;
    if (v < best) {
      best = v;
      grad[0] = g[0];
      grad[1] = g[1];
      grad[2] = g[2];
    }
  }
  return best;
}

enum { MODE_SUM = 0, MODE_MIN = 1 };

__device__ __forceinline__ int64_t clamp_wp(int64_t v, int64_t lo, int64_t hi) { return v < lo ? lo : (v > hi ? hi : v); }

struct CostArgs {
  int mode, pose_slot, qd;
  float w_pos, w_rot, w_col, margin, cutoff, w_smooth, lr;
  int steps, clamp;
  float lo[PM_GRAD_MAXQ], hi[PM_GRAD_MAXQ], dofw2[PM_GRAD_MAXQ];
};

// Cost of ws.q (returned on every lane) and, when WANT_GRAD, its gradient in ws.g.
// target: 7 floats (x y z qx qy qz qw) or null.
template <bool WANT_GRAD, int GW = 32>
__device__ float warp_cost(const Tab& t, const CostArgs& a, const WS& ws, const float* target, int lane) {
  warp_fk<GW>(t, ws, lane);
  // pose term (lane 0), wrench kept in misc[0..5]
  float cost = 0.f;
  if (lane == 0) {
    for (int k = 0; k < 6; k++) ws.misc[k] = 0.f;
    if (a.pose_slot >= 0 && target) {
      const float* w = ws.sw + (size_t)a.pose_slot * kSlotF;
      float e[3];
      for (int k = 0; k < 3; k++) e[k] = w[12 + k] - target[k];
      const FQ qt{target[3], target[4], target[5], target[6]};
      float phi[3];
      rotvec_error(FQ{w[8], w[9], w[10], w[11]}, qt, phi);
      cost = a.w_pos * fmaf(e[0], e[0], fmaf(e[1], e[1], e[2] * e[2])) + a.w_rot * fmaf(phi[0], phi[0], fmaf(phi[1], phi[1], phi[2] * phi[2]));
      float wp[3];
      fqrot(qt, phi, wp);
      for (int k = 0; k < 3; k++) {
        ws.misc[k] = 2.f * a.w_pos * e[k];
        ws.misc[3 + k] = 2.f * a.w_rot * wp[k];
      }
    }
  }
  // spheres; first, per slot, the primitives its bounding sphere leaves within thr (a sphere's
  // distance lower bound is at least its slot's), kept in the slot work's word 31
  const float thr = a.mode == MODE_MIN ? a.cutoff : a.margin;
  for (int i = lane; i < t.n_slots; i += GW) {
    const float4 b = t.sbnd[i];
    float* w = ws.sw + (size_t)i * kSlotF;
    unsigned m = 0;
    if (b.w >= 0.f && t.n_prims <= 32) {
      const float* R = w + 16;
      const float gx = fmaf(R[0], b.x, fmaf(R[1], b.y, fmaf(R[2], b.z, w[12])));
      const float gy = fmaf(R[3], b.x, fmaf(R[4], b.y, fmaf(R[5], b.z, w[13])));
      const float gz = fmaf(R[6], b.x, fmaf(R[7], b.y, fmaf(R[8], b.z, w[14])));
      for (int j = 0; j < t.n_prims; j++) {
        const GPrim& P = t.prim[j];
        // keep unless |gc - pos| >= thr + bound + R (squared, with 1e-5 relative to spare)
        const float sr = thr + P.bound + b.w;
        const float dx = gx - P.pos[0], dy = gy - P.pos[1], dz = gz - P.pos[2];
        const bool keep = P.bound < 0.f || (sr > 0.f && fmaf(dx, dx, fmaf(dy, dy, dz * dz)) < sr * sr * (1.f + 1e-5f));
        m |= keep ? 1u << j : 0u;
      }
    }
    w[31] = __uint_as_float(m);
  }
  __syncwarp();
  float best_d = INFINITY;
  int best_k = 0x7fffffff;
  float best_g[3] = {0.f, 0.f, 0.f};
  float hsum = 0.f;
  for (int k = lane; k < t.n_sph; k += GW) {
    const GSph& s = t.sph[k];
    const float* w = ws.sw + (size_t)s.slot * kSlotF;
    const float* R = w + 16;
    float c[3];
    c[0] = fmaf(R[0], s.x, fmaf(R[1], s.y, fmaf(R[2], s.z, w[12])));
    c[1] = fmaf(R[3], s.x, fmaf(R[4], s.y, fmaf(R[5], s.z, w[13])));
    c[2] = fmaf(R[6], s.x, fmaf(R[7], s.y, fmaf(R[8], s.z, w[14])));
    float g[3] = {0.f, 0.f, 0.f};
    float f[3] = {0.f, 0.f, 0.f};
    if (s.active) {
      const float d = sphere_min_dist(t, c, s.r, thr, g, __float_as_uint(w[31]));
      if (a.mode == MODE_SUM) {
        const float h = fmaxf(a.margin - d, 0.f);
        hsum = fmaf(h, h, hsum);
        const float sc = -2.f * a.w_col * h;
        f[0] = sc * g[0];
        f[1] = sc * g[1];
        f[2] = sc * g[2];
      } else if (d < best_d) {
        best_d = d;
        best_k = k;
        best_g[0] = g[0];
        best_g[1] = g[1];
        best_g[2] = g[2];
      }
    }
    if (WANT_GRAD) {
      float* sa = ws.sadj + (size_t)6 * k;
      const float rel[3] = {c[0] - w[12], c[1] - w[13], c[2] - w[14]};
      float m[3];
      cross3(rel, f, m);
      for (int q = 0; q < 3; q++) {
        sa[q] = f[q];
        sa[3 + q] = m[q];
      }
    }
  }
  if (a.mode == MODE_SUM) {
    cost += a.w_col * hsum;
    cost = warp_sum<GW>(cost);
  } else {
    // the unit's argmin over (d, sphere index); ties go to the lower index
    for (int o = GW / 2; o > 0; o >>= 1) {
      const float od = __shfl_xor_sync(0xffffffffu, best_d, o);
      const int ok = __shfl_xor_sync(0xffffffffu, best_k, o);
      if (od < best_d || (od == best_d && ok < best_k)) {
        best_d = od;
        best_k = ok;
      }
    }
    cost = fminf(best_d, a.cutoff);
    if (WANT_GRAD) {
      __syncwarp();
      if (best_d < a.cutoff && (best_k & (GW - 1)) == lane) {  // the owner seeds the adjoint with grad d
        const GSph& s = t.sph[best_k];
        const float* w = ws.sw + (size_t)s.slot * kSlotF;
        const float* R = w + 16;
        const float rel[3] = {fmaf(R[0], s.x, fmaf(R[1], s.y, R[2] * s.z)), fmaf(R[3], s.x, fmaf(R[4], s.y, R[5] * s.z)),
                              fmaf(R[6], s.x, fmaf(R[7], s.y, R[8] * s.z))};
        float m[3];
        cross3(rel, best_g, m);
        float* sa = ws.sadj + (size_t)6 * best_k;
        for (int q = 0; q < 3; q++) {
          sa[q] = best_g[q];
          sa[3 + q] = m[q];
        }
      }
    }
  }
  if (!WANT_GRAD) return cost;
  __syncwarp();
  // per-slot wrench (moment about the slot origin), plus the pose wrench
  for (int i = lane; i < t.n_slots; i += GW) {
    float F[3] = {0.f, 0.f, 0.f}, M[3] = {0.f, 0.f, 0.f};
    for (int k = t.sbeg[i]; k < t.sbeg[i + 1]; k++) {
      const float* sa = ws.sadj + (size_t)6 * k;
      for (int q = 0; q < 3; q++) {
        F[q] += sa[q];
        M[q] += sa[3 + q];
      }
    }
    if (i == a.pose_slot) {
      for (int q = 0; q < 3; q++) {
        F[q] += ws.misc[q];
        M[q] += ws.misc[3 + q];
      }
    }
    float* w = ws.sw + (size_t)i * kSlotF;
    for (int q = 0; q < 3; q++) {
      w[25 + q] = F[q];
      w[28 + q] = M[q];
    }
  }
  for (int j = lane; j < t.qd; j += GW) ws.g[j] = 0.f;
  __syncwarp();
  if (t.n_slots <= GW && g_tree_bad == 0) {
    // subtree totals on the unit's lanes, one slot each: with moments taken about the world origin
    // (M + o x F) a subtree's wrench is a plain sum, and a subtree is the slot range [i, send), so
    // an inclusive prefix sum over the lanes gives every total at once; the moment is then moved
    // back to the slot's origin (M_sub - o x F_sub)
    const unsigned FULL = 0xffffffffu;
    const int i = lane;
    const bool own = i < t.n_slots;
    float v[6] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f}, o[3] = {0.f, 0.f, 0.f};
    if (own) {
      const float* w = ws.sw + (size_t)i * kSlotF;
      for (int k = 0; k < 3; k++) {
        o[k] = w[12 + k];
        v[k] = w[25 + k];
      }
      float m[3];
      cross3(o, v, m);
      for (int k = 0; k < 3; k++) v[3 + k] = w[28 + k] + m[k];
    }
    for (int d = 1; d < GW; d <<= 1)
      for (int k = 0; k < 6; k++) {
        const float u = __shfl_up_sync(FULL, v[k], d, GW);
        if (i >= d) v[k] += u;
      }
    const int e = own ? t.slot[i].send - 1 : i;
    float sub[6];
    for (int k = 0; k < 6; k++) {
      const float hi = __shfl_sync(FULL, v[k], e, GW), lo = __shfl_sync(FULL, v[k], i > 0 ? i - 1 : 0, GW);
      sub[k] = i > 0 ? hi - lo : hi;
    }
    if (own) {
      float* w = ws.sw + (size_t)i * kSlotF;
      float m[3];
      cross3(o, sub, m);
      for (int k = 0; k < 3; k++) {
        w[25 + k] = sub[k];
        w[28 + k] = sub[3 + k] - m[k];
      }
    }
  } else if (lane == 0) {  // children first: move each subtree wrench to the parent origin
    for (int i = t.n_slots - 1; i >= 0; i--) {
      const int p = t.slot[i].parent;
      if (p < 0) continue;
      float* w = ws.sw + (size_t)i * kSlotF;
      float* pw = ws.sw + (size_t)p * kSlotF;
      const float arm[3] = {w[12] - pw[12], w[13] - pw[13], w[14] - pw[14]};
      float m[3];
      cross3(arm, w + 25, m);
      for (int q = 0; q < 3; q++) {
        pw[25 + q] += w[25 + q];
        pw[28 + q] += w[28 + q] + m[q];
      }
    }
  }
  __syncwarp();
  for (int i = lane; i < t.n_slots; i += GW) {
    const GSlot& s = t.slot[i];
    const float* w = ws.sw + (size_t)i * kSlotF;
    if (s.parent < 0) {
      const float* F = w + 25;
      const float* M = w + 28;
      float* g = ws.g + t.n_ctrl;
      if (t.base_type == PM_BASE_PLANAR) {
        g[0] = F[0];
        g[1] = F[1];
        g[2] = M[2];
      } else if (t.base_type == PM_BASE_FLOATING) {
        // q = R_z(yaw) R_y(pitch) R_x(roll): angular velocity axes of the three angles
        float sp, cp, sy, cy;
        sincosf(ws.q[t.n_ctrl + 4], &sp, &cp);
        sincosf(ws.q[t.n_ctrl + 5], &sy, &cy);
        g[0] = F[0];
        g[1] = F[1];
        g[2] = F[2];
        g[3] = fmaf(cy * cp, M[0], fmaf(sy * cp, M[1], -sp * M[2]));
        g[4] = fmaf(-sy, M[0], cy * M[1]);
        g[5] = M[2];
      }
      continue;
    }
    if (s.mode == PM_FK_STATE) continue;
    const float* R = w + 16;
    const float ax[3] = {fmaf(R[0], s.axis[0], fmaf(R[1], s.axis[1], R[2] * s.axis[2])),
                         fmaf(R[3], s.axis[0], fmaf(R[4], s.axis[1], R[5] * s.axis[2])),
                         fmaf(R[6], s.axis[0], fmaf(R[7], s.axis[1], R[8] * s.axis[2]))};
    const float* v = s.mode == PM_FK_PRIS ? w + 25 : w + 28;
    ws.g[s.qcol] = fmaf(ax[0], v[0], fmaf(ax[1], v[1], ax[2] * v[2]));
  }
  __syncwarp();
  return cost;
}

// ---------------------------------------------------------------------------------- IK batch
// lanes per problem and the blocks per SM the registers are sized for: 16 lanes at 4 blocks of 256
// threads (64 registers) keep all 8,192 problems of the 7-joint IK workload resident at once and
// measured fastest, ahead of 16 lanes at 2 or 3 blocks and of a whole warp per problem
constexpr int kIkGW = 16, kIkBlocksPerSm = 4;
// GW lanes per problem, 32 / GW problems per warp (the FK composition and the wrench accumulation,
// which run on one lane per problem, then serve that many problems at a time).  The loop over a
// warp's problems runs the same number of times on every group of the warp; a group past the end
// works on a copy of the last problem and writes nothing.
template <bool WANT_GRAD, int GW>
__global__ void __launch_bounds__(kNW * 32, kIkBlocksPerSm) k_ik_cost(const PmTablesHdr* __restrict__ T, const double* __restrict__ state, CostArgs a,
                                                      Layout L, float* __restrict__ q, const float* __restrict__ target, int64_t B,
                                                      float* __restrict__ cost, float* __restrict__ grad, float* __restrict__ hist) {
  extern __shared__ __align__(16) char smem[];
  Tab t;
  stage(T, state, L, smem, t);
  constexpr int per_warp = 32 / GW, groups = kNW * per_warp;
  const int lane = threadIdx.x & (GW - 1), gi = threadIdx.x / GW;
  const int first = (threadIdx.x >> 5) * per_warp;  // the warp's first group
  WS ws = warp_ws(L, smem, gi);
  for (int64_t u0 = (int64_t)blockIdx.x * groups + first; u0 < B; u0 += (int64_t)gridDim.x * groups) {
    const int64_t u_own = u0 + (gi - first);
    const bool have = u_own < B;
    const int64_t u = have ? u_own : B - 1;
    for (int j = lane; j < a.qd; j += GW) ws.q[j] = q[u * a.qd + j];
    __syncwarp();
    const float* tg = target ? target + u * 7 : nullptr;
    if (a.steps <= 0) {  // one evaluation
      const float c = warp_cost<WANT_GRAD, GW>(t, a, ws, tg, lane);
      if (have && lane == 0 && cost) cost[u] = c;
      if (WANT_GRAD && have)
        for (int j = lane; j < a.qd; j += GW) grad[u * a.qd + j] = ws.g[j];
      __syncwarp();
      continue;
    }
    // gradient descent, all steps in registers/shared memory: q <- clamp(q - lr * grad)
    for (int it = 0; it < a.steps; it++) {
      const float c = warp_cost<true, GW>(t, a, ws, tg, lane);
      if (have && lane == 0 && hist) hist[u * a.steps + it] = c;
      for (int j = lane; j < a.qd; j += GW) {
        float v = fmaf(-a.lr, ws.g[j], ws.q[j]);
        if (a.clamp) v = fminf(fmaxf(v, a.lo[j]), a.hi[j]);
        ws.q[j] = v;
      }
      __syncwarp();
    }
    if (cost) {
      const float c = warp_cost<false, GW>(t, a, ws, tg, lane);
      if (have && lane == 0) cost[u] = c;
    }
    if (have)
      for (int j = lane; j < a.qd; j += GW) q[u * a.qd + j] = ws.q[j];
    __syncwarp();
  }
}

// -------------------------------------------------------------------------- trajectory batch
// lanes per waypoint: a whole warp measured 12 % faster than half warps on the 512-trajectory
// planar-chain workload (the cloud queries of a half warp's spheres diverge more)
constexpr int kTrajGW = 32;
// GW lanes per waypoint: 32 (one waypoint per warp) or 16 (two per warp, a half each, as in
// k_ik_cost).  wp_cost[u] = collision hinge of waypoint u plus, for interior waypoints, the
// smoothness term of its acceleration; grad row u when requested.
// Up to 85 registers (3 blocks of 256 threads per SM).
template <bool WANT_GRAD, int GW>
__global__ void __launch_bounds__(kNW * 32, 3) k_traj_cost(const PmTablesHdr* __restrict__ T, const double* __restrict__ state, CostArgs a,
                                                        Layout L, const float* __restrict__ q, const int64_t* __restrict__ off,
                                                        int64_t n_traj, int64_t n_wp, float* __restrict__ wp_cost,
                                                        float* __restrict__ grad) {
  extern __shared__ __align__(16) char smem[];
  Tab t;
  stage(T, state, L, smem, t);
  constexpr int per_warp = 32 / GW, groups = kNW * per_warp;
  const int lane = threadIdx.x & (GW - 1), gi = threadIdx.x / GW;
  const int first = (threadIdx.x >> 5) * per_warp;
  WS ws = warp_ws(L, smem, gi);
  const int d = a.qd;
  for (int64_t u0 = (int64_t)blockIdx.x * groups + first; u0 < n_wp; u0 += (int64_t)gridDim.x * groups) {
    const int64_t u_own = u0 + (gi - first);
    const bool have = u_own < n_wp;  // a half past the end works on a copy of the last waypoint, writes nothing
    const int64_t u = have ? u_own : n_wp - 1;
    // trajectory of u: the last i with off[i] <= u
    int64_t lo = 0, hi = n_traj;
    while (hi - lo > 1) {
      const int64_t mid = (lo + hi) >> 1;
      if (off[mid] <= u) lo = mid;
      else hi = mid;
    }
    const int64_t b = clamp_wp(off[lo], 0, n_wp), e = clamp_wp(off[lo + 1], b, n_wp);
    for (int j = lane; j < d; j += GW) ws.q[j] = q[u * d + j];
    __syncwarp();
    float c = warp_cost<WANT_GRAD, GW>(t, a, ws, nullptr, lane);
    // smoothness: acc(k) = q[k+1] - 2 q[k] + q[k-1] for b < k < e-1
    auto acc = [&](int64_t k, int j) -> float {
      if (k <= b || k >= e - 1) return 0.f;
      return q[(k + 1) * d + j] - 2.f * q[k * d + j] + q[(k - 1) * d + j];
    };
    float sm = 0.f;
    for (int j = lane; j < d; j += GW) {
      const float ac = acc(u, j);
      sm = fmaf(a.dofw2[j] * ac, ac, sm);
      if (WANT_GRAD && have) {
        const float gs = 2.f * a.w_smooth * a.dofw2[j] * (acc(u - 1, j) - 2.f * ac + acc(u + 1, j));
        grad[u * d + j] = ws.g[j] + gs;
      }
    }
    c += a.w_smooth * warp_sum<GW>(sm);
    if (have && lane == 0) wp_cost[u] = c;
    __syncwarp();
  }
}

// cost[i] = sum of wp_cost over trajectory i, in a fixed order (one warp per trajectory).
__global__ void __launch_bounds__(256) k_traj_sum(const int64_t* __restrict__ off, int64_t n_traj, int64_t n_wp, const float* __restrict__ wp_cost,
                           float* __restrict__ cost) {
  const int lane = threadIdx.x & 31;
  const int64_t i = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  if (i >= n_traj) return;
  const int64_t b = clamp_wp(off[i], 0, n_wp), e = clamp_wp(off[i + 1], b, n_wp);
  float s = 0.f;
  for (int64_t k = b + lane; k < e; k += 32) s += wp_cost[k];
  s = warp_sum(s);
  if (lane == 0) cost[i] = s;
}

// ------------------------------------------------------------------------- FP64 link poses
__global__ void k_link_pose64(const PmTablesHdr* __restrict__ T, const double* __restrict__ state, const double* __restrict__ q,
                              int64_t B, int slot, double* __restrict__ out7) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= B) return;
  struct Poses {
    DPose p[PM_MAX_SLOTS];
    __device__ DPose& operator[](int k) { return p[k]; }
  } P;
  fk64(T, state, q + i * T->q_dim, false, P);
  const DPose& r = P[slot];
  double* o = out7 + i * 7;
  o[0] = r.t.x;
  o[1] = r.t.y;
  o[2] = r.t.z;
  o[3] = r.q.x;
  o[4] = r.q.y;
  o[5] = r.q.z;
  o[6] = r.q.w;
}

CostArgs to_args(const pmg::GradArgs& g, int qd) {
  CostArgs a;
  a.mode = g.mode;
  a.pose_slot = g.pose_slot;
  a.qd = qd;
  a.w_pos = g.w_pos;
  a.w_rot = g.w_rot;
  a.w_col = g.w_col;
  a.margin = g.margin;
  a.cutoff = g.cutoff;
  a.w_smooth = g.w_smooth;
  a.lr = g.lr;
  a.steps = g.steps;
  a.clamp = g.clamp;
  for (int j = 0; j < PM_GRAD_MAXQ; j++) {
    a.lo[j] = g.lo[j];
    a.hi[j] = g.hi[j];
    a.dofw2[j] = g.dofw2[j];
  }
  return a;
}

int grid_for(const void* fn, size_t smem, int64_t units, int per_block = kNW) {
  int dev = 0, n_sm = 0, per_sm = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&n_sm, cudaDevAttrMultiProcessorCount, dev);
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, kNW * 32, smem);
  const int64_t need = (units + per_block - 1) / per_block;
  return (int)std::max<int64_t>(1, std::min<int64_t>(need, (int64_t)std::max(per_sm, 1) * n_sm));
}

template <class K>
cudaError_t prep(K fn, size_t smem) {
  if (smem > 48 * 1024) {
    cudaError_t e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
  }
  return cudaSuccess;
}

}  // namespace

namespace pmg {

size_t grad_smem_bytes(const PmTablesHdr& h) { return make_layout(h.n_slots, h.n_spheres, h.n_prims, h.q_dim).total; }

cudaError_t launch_ik_cost(const PmTablesHdr* T, const PmTablesHdr& h, const double* state, const GradArgs& g, float* q,
                           const float* target, int64_t B, float* cost, float* grad, float* hist, cudaStream_t s) {
  if (B <= 0) return cudaSuccess;
  constexpr int GW = kIkGW, groups = kNW * (32 / GW);
  Layout L = make_layout(h.n_slots, h.n_spheres, h.n_prims, h.q_dim, groups);
  L.n_ctrl = h.n_ctrl;
  L.base_type = h.base_type;
  L.off_clouds = h.off_clouds;
  const CostArgs a = to_args(g, h.q_dim);
  if (grad || g.steps > 0) {
    auto fn = k_ik_cost<true, GW>;
    cudaError_t e = prep(fn, L.total);
    if (e != cudaSuccess) return e;
    prof_begin("k_ik_cost", s);
    fn<<<grid_for((const void*)fn, L.total, B, groups), kNW * 32, L.total, s>>>(T, state, a, L, q, target, B, cost, grad, hist);
    prof_end("k_ik_cost", s);
  } else {
    auto fn = k_ik_cost<false, GW>;
    cudaError_t e = prep(fn, L.total);
    if (e != cudaSuccess) return e;
    fn<<<grid_for((const void*)fn, L.total, B, groups), kNW * 32, L.total, s>>>(T, state, a, L, q, target, B, cost, nullptr, nullptr);
  }
  return cudaGetLastError();
}

cudaError_t launch_traj_cost(const PmTablesHdr* T, const PmTablesHdr& h, const double* state, const GradArgs& g, const float* q,
                             const int64_t* off, int64_t n_traj, int64_t n_wp, float* wp_cost, float* cost, float* grad,
                             cudaStream_t s) {
  if (n_traj <= 0) return cudaSuccess;
  constexpr int GW = kTrajGW, groups = kNW * (32 / GW);
  Layout L = make_layout(h.n_slots, h.n_spheres, h.n_prims, h.q_dim, groups);
  L.n_ctrl = h.n_ctrl;
  L.base_type = h.base_type;
  L.off_clouds = h.off_clouds;
  const CostArgs a = to_args(g, h.q_dim);
  if (n_wp > 0) {
    if (grad) {
      auto fn = k_traj_cost<true, GW>;
      cudaError_t e = prep(fn, L.total);
      if (e != cudaSuccess) return e;
      prof_begin("k_traj_cost", s);
      fn<<<grid_for((const void*)fn, L.total, n_wp, groups), kNW * 32, L.total, s>>>(T, state, a, L, q, off, n_traj, n_wp, wp_cost, grad);
      prof_end("k_traj_cost", s);
    } else {
      auto fn = k_traj_cost<false, GW>;
      cudaError_t e = prep(fn, L.total);
      if (e != cudaSuccess) return e;
      fn<<<grid_for((const void*)fn, L.total, n_wp, groups), kNW * 32, L.total, s>>>(T, state, a, L, q, off, n_traj, n_wp, wp_cost, nullptr);
    }
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
  }
  const int64_t threads = n_traj * 32;
  k_traj_sum<<<(unsigned)((threads + 255) / 256), 256, 0, s>>>(off, n_traj, n_wp, wp_cost, cost);
  return cudaGetLastError();
}

cudaError_t launch_link_pose64(const PmTablesHdr* T, const double* state, const double* q, int64_t B, int slot, double* out7,
                               cudaStream_t s) {
  if (B <= 0) return cudaSuccess;
  k_link_pose64<<<(unsigned)((B + 127) / 128), 128, 0, s>>>(T, state, q, B, slot, out7);
  return cudaGetLastError();
}

}  // namespace pmg
