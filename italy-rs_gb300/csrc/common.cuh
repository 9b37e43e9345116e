// Device-side building blocks shared by the bake kernels (sm_103a).
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

namespace sdfb {

// ---------------------------------------------------------------------------------------------
// Error flags raised by kernels (OR-ed into one device word, read by the host after a bake).
enum DevErr : uint32_t {
  kErrBadIndex = 1u,          // triangle index >= V
  kErrNonFinite = 2u,         // vertex with NaN / Inf coordinate
  kErrStackOverflow = 4u,     // traversal stack exhausted
  kErrCrossingOverflow = 8u,  // parity crossing list exceeded its capacity
  kErrEmpty = 16u,
  kErrCorruptTree = 32u,      // a node or leaf reference out of range, or a walk that never ends
  kErrDispatch = 64u,         // a block's tile dispatch waited past its limit
};

// sdfb_opts.fault_inject bits as the kernels see them (include/sdfb.h, SDFB_FAULT_*).
enum FaultBits : int { kFaultDispatch = 1, kFaultStepLimit = 2, kFaultShallowStack = 4, kFaultStackAll = 8 };

constexpr int kWarp = 32;
constexpr uint32_t kFull = 0xffffffffu;

// ---------------------------------------------------------------------------------------------
// Cell centre, exactly as the reference rounds it: origin + (float(i) + 0.5f) * voxel, with no
// fused multiply-add (src/convert/sdf_baker.cpp:107, src/render/kernels/sdf_bake.cu:34-37).
__device__ __forceinline__ float cell_center(float origin, int i, float voxel) {
  return __fadd_rn(origin, __fmul_rn(__fadd_rn(__int2float_rn(i), 0.5f), voxel));
}

// float -> int after floor, saturating, NaN -> 0 (cvt.rzi.s32.f32).
__device__ __forceinline__ int f2i_sat(float f) { return __float2int_rz(f); }

__device__ __forceinline__ int clampi(int v, int lo, int hi) { return v < lo ? lo : (v > hi ? hi : v); }

// std::min / std::max as the reference evaluates them.
__device__ __forceinline__ float min_ref(float a, float b) { return (b < a) ? b : a; }
__device__ __forceinline__ float max_ref(float a, float b) { return (a < b) ? b : a; }

// ---------------------------------------------------------------------------------------------
// Triangle / box separating-axis test with the reference's exact FP32 rounding
// (src/convert/tri_box_overlap.h:12-114): every product and sum is one IEEE operation, in the
// reference's order, through the _rn intrinsics so that nothing contracts into an FMA. The
// occupancy it defines must match the reference bit for bit.
struct f3 {
  float x, y, z;
};

__device__ __forceinline__ f3 sub3(f3 a, f3 b) { return {__fsub_rn(a.x, b.x), __fsub_rn(a.y, b.y), __fsub_rn(a.z, b.z)}; }
__device__ __forceinline__ float mul(float a, float b) { return __fmul_rn(a, b); }

__device__ __forceinline__ bool axis_overlaps(float pa, float pb, float rad) {
  const float mn = min_ref(pa, pb), mx = max_ref(pa, pb);
  return !(mn > rad || mx < -rad);
}
// Edge (a, b) projections onto e x X, e x Y, e x Z in the reference's operand pairing.
__device__ __forceinline__ float proj_x(float a, float b, f3 v) { return __fsub_rn(mul(a, v.y), mul(b, v.z)); }
__device__ __forceinline__ float proj_y(float a, float b, f3 v) { return __fadd_rn(mul(-a, v.x), mul(b, v.z)); }
__device__ __forceinline__ float proj_z(float a, float b, f3 v) { return __fsub_rn(mul(a, v.x), mul(b, v.y)); }
__device__ __forceinline__ float rad2(float fa, float ha, float fb, float hb) { return __fadd_rn(mul(fa, ha), mul(fb, hb)); }
__device__ __forceinline__ float dot_ref(f3 a, f3 b) {
  return __fadd_rn(__fadd_rn(mul(a.x, b.x), mul(a.y, b.y)), mul(a.z, b.z));
}

__device__ __forceinline__ bool plane_box_overlap(f3 n, f3 v, float h) {
  f3 vmin, vmax;
  vmin.x = n.x > 0.0f ? __fsub_rn(-h, v.x) : __fsub_rn(h, v.x);
  vmax.x = n.x > 0.0f ? __fsub_rn(h, v.x) : __fsub_rn(-h, v.x);
  vmin.y = n.y > 0.0f ? __fsub_rn(-h, v.y) : __fsub_rn(h, v.y);
  vmax.y = n.y > 0.0f ? __fsub_rn(h, v.y) : __fsub_rn(-h, v.y);
  vmin.z = n.z > 0.0f ? __fsub_rn(-h, v.z) : __fsub_rn(h, v.z);
  vmax.z = n.z > 0.0f ? __fsub_rn(h, v.z) : __fsub_rn(-h, v.z);
  if (dot_ref(n, vmin) > 0.0f) return false;
  return dot_ref(n, vmax) >= 0.0f;
}

// Box centre c, cubic half extent h (the reference always passes vec3(voxel * 0.5f)).
__device__ __forceinline__ bool sat_overlap(f3 c, float h, f3 t0, f3 t1, f3 t2) {
  const f3 v0 = sub3(t0, c), v1 = sub3(t1, c), v2 = sub3(t2, c);
  const f3 e0 = sub3(v1, v0), e1 = sub3(v2, v1), e2 = sub3(v0, v2);
  float fx = fabsf(e0.x), fy = fabsf(e0.y), fz = fabsf(e0.z);
  if (!axis_overlaps(proj_x(e0.z, e0.y, v0), proj_x(e0.z, e0.y, v2), rad2(fz, h, fy, h))) return false;
  if (!axis_overlaps(proj_y(e0.z, e0.x, v0), proj_y(e0.z, e0.x, v2), rad2(fz, h, fx, h))) return false;
  if (!axis_overlaps(proj_z(e0.y, e0.x, v1), proj_z(e0.y, e0.x, v2), rad2(fy, h, fx, h))) return false;
  fx = fabsf(e1.x); fy = fabsf(e1.y); fz = fabsf(e1.z);
  if (!axis_overlaps(proj_x(e1.z, e1.y, v0), proj_x(e1.z, e1.y, v2), rad2(fz, h, fy, h))) return false;
  if (!axis_overlaps(proj_y(e1.z, e1.x, v0), proj_y(e1.z, e1.x, v2), rad2(fz, h, fx, h))) return false;
  if (!axis_overlaps(proj_z(e1.y, e1.x, v0), proj_z(e1.y, e1.x, v1), rad2(fy, h, fx, h))) return false;
  fx = fabsf(e2.x); fy = fabsf(e2.y); fz = fabsf(e2.z);
  if (!axis_overlaps(proj_x(e2.z, e2.y, v0), proj_x(e2.z, e2.y, v1), rad2(fz, h, fy, h))) return false;
  if (!axis_overlaps(proj_y(e2.z, e2.x, v0), proj_y(e2.z, e2.x, v1), rad2(fz, h, fx, h))) return false;
  if (!axis_overlaps(proj_z(e2.y, e2.x, v1), proj_z(e2.y, e2.x, v2), rad2(fy, h, fx, h))) return false;
  if (min_ref(min_ref(v0.x, v1.x), v2.x) > h || max_ref(max_ref(v0.x, v1.x), v2.x) < -h) return false;
  if (min_ref(min_ref(v0.y, v1.y), v2.y) > h || max_ref(max_ref(v0.y, v1.y), v2.y) < -h) return false;
  if (min_ref(min_ref(v0.z, v1.z), v2.z) > h || max_ref(max_ref(v0.z, v1.z), v2.z) < -h) return false;
  const f3 n = {__fsub_rn(mul(e0.y, e1.z), mul(e1.y, e0.z)), __fsub_rn(mul(e0.z, e1.x), mul(e1.z, e0.x)),
                __fsub_rn(mul(e0.x, e1.y), mul(e1.x, e0.y))};
  return plane_box_overlap(n, v0, h);
}

// Candidate cell range of a triangle along one axis: floor((min - origin) / voxel) clamped to
// [0, nmax] (sdf_baker.cpp:97-101), IEEE division, saturating conversion.
__device__ __forceinline__ int cell_index_clamped(float c, float origin, float voxel, int nmax) {
  return clampi(f2i_sat(floorf(__fdiv_rn(__fsub_rn(c, origin), voxel))), 0, nmax);
}

// ---------------------------------------------------------------------------------------------
// Exact 2-D orientation with simulation of simplicity (parity sign).
//
// orient(a, b, p) = (b - a) x (p - a) for FP32 inputs. A FP32 evaluation is accepted when its
// magnitude exceeds a forward error bound (Shewchuk 1997, the orient2d "A" bound with a safety
// margin); otherwise the value is expanded into six products of inputs, each exact in FP64, and
// the sign of their sum is found exactly with Two-Sum / Grow-Expansion. A zero value is broken as
// if p were p + (eps, eps^2): the sign becomes that of (a_v - b_v), else (b_u - a_u).

__device__ __forceinline__ void two_sum(double a, double b, double &s, double &e) {
  const double x = __dadd_rn(a, b);
  const double bv = __dsub_rn(x, a);
  const double av = __dsub_rn(x, bv);
  s = x;
  e = __dadd_rn(__dsub_rn(a, av), __dsub_rn(b, bv));
}

static __device__ __noinline__ int exact_orient_sign(float au, float av, float bu, float bv, float pu, float pv) {
  double t[6];
  t[0] = __dmul_rn((double)bu, (double)pv);
  t[1] = -__dmul_rn((double)bu, (double)av);
  t[2] = -__dmul_rn((double)au, (double)pv);
  t[3] = -__dmul_rn((double)bv, (double)pu);
  t[4] = __dmul_rn((double)bv, (double)au);
  t[5] = __dmul_rn((double)av, (double)pu);
  double e[6];
  int m = 1;
  e[0] = t[0];
#pragma unroll
  for (int k = 1; k < 6; ++k) {
    double q = t[k];
#pragma unroll
    for (int i = 0; i < 6; ++i) {
      if (i < m) {
        double s, err;
        two_sum(q, e[i], s, err);
        e[i] = err;
        q = s;
      }
    }
    e[m++] = q;
  }
  int sign = 0;
#pragma unroll
  for (int i = 0; i < 6; ++i)
    if (e[i] != 0.0) sign = e[i] > 0.0 ? 1 : -1;  // last non-zero = most significant
  return sign;
}

// Returns the orientation sign (+1 / -1) and the FP32 value (for barycentric weights).
__device__ __forceinline__ int orient2_sos(float au, float av, float bu, float bv, float pu, float pv, float &val) {
  const float l = __fmul_rn(__fsub_rn(bu, au), __fsub_rn(pv, av));
  const float r = __fmul_rn(__fsub_rn(bv, av), __fsub_rn(pu, au));
  const float det = __fsub_rn(l, r);
  val = det;
  const float bound = 4.0f * 5.9604645e-8f * (fabsf(l) + fabsf(r));  // 4 * 2^-24 * (|l| + |r|)
  if (fabsf(det) > bound && fabsf(det) > 1e-30f) return det > 0.0f ? 1 : -1;
  const int s = exact_orient_sign(au, av, bu, bv, pu, pv);
  if (s) return s;
  if (av != bv) return av > bv ? 1 : -1;
  if (bu != au) return bu > au ? 1 : -1;
  return 0;
}

// Does the +z line through (px, py) cross triangle (a, b, c)? On a crossing *z receives the
// crossing height (FP32 barycentric blend, within the triangle's z range) and *s the crossing's
// orientation: +1 when the triangle winds counter-clockwise seen from +z (its normal has a
// positive z component, so the ray leaves an outward-oriented closed surface there), else -1.
__device__ __forceinline__ bool column_crossing(f3 a, f3 b, f3 c, float px, float py, float &z, int &s) {
  float wab, wbc, wca;
  const int s0 = orient2_sos(a.x, a.y, b.x, b.y, px, py, wab);
  if (s0 == 0) return false;
  const int s1 = orient2_sos(b.x, b.y, c.x, c.y, px, py, wbc);
  if (s1 != s0) return false;
  const int s2 = orient2_sos(c.x, c.y, a.x, a.y, px, py, wca);
  if (s2 != s0) return false;
  const float wa = fabsf(wbc), wb = fabsf(wca), wc = fabsf(wab);
  const float den = wa + wb + wc;
  if (den > 0.0f) {
    z = (wa * a.z + wb * b.z + wc * c.z) / den;
    z = fminf(fmaxf(z, fminf(fminf(a.z, b.z), c.z)), fmaxf(fmaxf(a.z, b.z), c.z));
  } else {
    z = (a.z + b.z + c.z) * (1.0f / 3.0f);
  }
  s = s0;
  return true;
}

// ---------------------------------------------------------------------------------------------
// Triangle record of the winding-number hierarchy: 64 bytes, four float4s, in BVH leaf order.
//   r0 = (v0, 1/|e1|^2)    e1 = v1 - v0
//   r1 = (e1, 1/|e2|^2)    e2 = v2 - v0
//   r2 = (e2, 1/|e3|^2)    e3 = v2 - v1
//   r3 = (n,  |n|)         n = e1 x e2 (|n| is twice the area)
struct TriRec {
  float4 r0, r1, r2, r3;
};

__device__ __forceinline__ float inv_or_zero(float x) { return x > 0.0f ? 1.0f / x : 0.0f; }

// ---------------------------------------------------------------------------------------------
// Triangle record for distance queries: 80 bytes, five float4s, in BVH leaf order. Each triangle
// is stored in its own orthonormal frame: origin at vertex A, u along the longest edge AB, v in
// the triangle's plane towards C, h along the unit normal. In that frame the triangle is
// A = (0, 0), B = (b, 0), C = (c1, c2) with c2 >= 0 and 0 <= c1 <= b.
//   q0 = (A, b)
//   q1 = (e_u, c1)
//   q2 = (e_v, c2)
//   q3 = (e_h, c1 - b)
//   q4 = (c1 / |AC|^2, c2 / |AC|^2, (c1 - b) / |BC|^2, c2 / |BC|^2)   (0 for a zero-length edge)
// A point's squared distance is h^2 plus the squared in-plane distance from (u, v) to the 2D
// triangle: zero inside it, else the nearest of the three clamped edge projections. A collinear
// or point-like triangle has c2 = 0 and is never inside (the inside test is strict), so only its
// edges count, and with c2 = 0 those are pieces of the u axis. The frame is computed in FP64 from
// the FP32 vertices and then rounded; A is the exact input vertex.
//
// The frame makes a query cheap where the traversal spends its time: a lane holds several cells
// of one (x, y) column, so the x and y parts of u, v and h are formed once per lane and each cell
// adds its z term with one FMA; the plane bound h^2 used to skip a triangle is the first step of
// the full test rather than extra work.
struct DistTri {
  float4 q0, q1, q2, q3, q4;
};

// Distance from u to [0, b] (edge AB's extent on the u axis).
__device__ __forceinline__ float dist_to_range(float u, float b) { return fmaxf(fmaxf(-u, u - b), 0.0f); }

// Squared distance from (u, v) to the 2D triangle (0, 0), (b, 0), (c1, c2) of a DistTri, given
// du = dist_to_range(u, b) (q4 holds the edge projection factors). Branch-free: every lane
// executes the same instructions.
__device__ __forceinline__ float inplane_dist2(float u, float v, float du, float b, float c1, float c2, float bc,
                                               const float4 &k) {
  const float d_ab = fmaf(du, du, v * v);  // edge AB on the u axis
  const float s1 = __saturatef(fmaf(v, k.y, u * k.x));  // edge AC
  const float x1 = fmaf(-s1, c1, u), y1 = fmaf(-s1, c2, v);
  const float d_ac = fmaf(x1, x1, y1 * y1);
  const float ub = u - b;  // edge BC
  const float s2 = __saturatef(fmaf(v, k.w, ub * k.z));
  const float x2 = fmaf(-s2, bc, ub), y2 = fmaf(-s2, c2, v);
  const float d_bc = fmaf(x2, x2, y2 * y2);
  const bool inside = (v > 0.0f) & (fmaf(c2, u, -c1 * v) > 0.0f) & (fmaf(bc, v, -c2 * ub) > 0.0f);
  return inside ? 0.0f : fminf(fminf(d_ab, d_ac), d_bc);
}

// The DistTri of triangle (a, b, c), built in FP64.
__device__ inline DistTri make_dist_tri(float3 fa, float3 fb, float3 fc) {
  struct D3 {
    double x, y, z;
  };
  auto sub = [](D3 p, D3 q) { return D3{p.x - q.x, p.y - q.y, p.z - q.z}; };
  auto dot = [](D3 p, D3 q) { return p.x * q.x + p.y * q.y + p.z * q.z; };
  auto cross = [](D3 p, D3 q) { return D3{p.y * q.z - p.z * q.y, p.z * q.x - p.x * q.z, p.x * q.y - p.y * q.x}; };
  auto scale = [](D3 p, double s) { return D3{p.x * s, p.y * s, p.z * s}; };
  D3 v[3] = {{fa.x, fa.y, fa.z}, {fb.x, fb.y, fb.z}, {fc.x, fc.y, fc.z}};
  // Rotate the vertices so that AB is the longest edge (C then projects inside [A, B]).
  const double l0 = dot(sub(v[1], v[0]), sub(v[1], v[0]));  // v0 v1
  const double l1 = dot(sub(v[2], v[1]), sub(v[2], v[1]));  // v1 v2
  const double l2 = dot(sub(v[0], v[2]), sub(v[0], v[2]));  // v2 v0
  const int r = (l0 >= l1 && l0 >= l2) ? 0 : (l1 >= l2 ? 1 : 2);
  const D3 A = v[r], B = v[(r + 1) % 3], C = v[(r + 2) % 3];
  const D3 ab = sub(B, A), ac = sub(C, A);
  const double b = sqrt(dot(ab, ab));
  D3 eu{1.0, 0.0, 0.0}, ev{0.0, 1.0, 0.0};
  double c1 = 0.0, c2 = 0.0;
  if (b > 0.0) {
    eu = scale(ab, 1.0 / b);
    c1 = dot(ac, eu);
    const D3 perp = sub(ac, scale(eu, c1));
    c2 = sqrt(dot(perp, perp));
    if (c2 > 1e-12 * b) {
      ev = scale(perp, 1.0 / c2);
    } else {
      // Collinear: any unit vector perpendicular to e_u (from the axis e_u is least aligned with).
      c2 = 0.0;
      const double ax = fabs(eu.x), ay = fabs(eu.y), az = fabs(eu.z);
      const D3 axis = (ax <= ay && ax <= az) ? D3{1.0, 0.0, 0.0} : (ay <= az ? D3{0.0, 1.0, 0.0} : D3{0.0, 0.0, 1.0});
      const D3 w = sub(axis, scale(eu, dot(axis, eu)));
      ev = scale(w, 1.0 / sqrt(dot(w, w)));
    }
  }
  const D3 eh = cross(eu, ev);
  const double bc = c1 - b;
  const double ac2 = c1 * c1 + c2 * c2, bc2 = bc * bc + c2 * c2;
  const float3 fA = r == 0 ? fa : (r == 1 ? fb : fc);
  DistTri t;
  t.q0 = make_float4(fA.x, fA.y, fA.z, float(b));
  t.q1 = make_float4(float(eu.x), float(eu.y), float(eu.z), float(c1));
  t.q2 = make_float4(float(ev.x), float(ev.y), float(ev.z), float(c2));
  t.q3 = make_float4(float(eh.x), float(eh.y), float(eh.z), float(bc));
  t.q4 = make_float4(ac2 > 0.0 ? float(c1 / ac2) : 0.0f, ac2 > 0.0 ? float(c2 / ac2) : 0.0f,
                     bc2 > 0.0 ? float(bc / bc2) : 0.0f, bc2 > 0.0 ? float(c2 / bc2) : 0.0f);
  return t;
}

// FP32 arithmetic of the distance tests as the kernel executes it, counted as flops (add / sub /
// mul = 1, FMA = 2; min, max, saturate and compares are not counted), for the roofline figure.
// The work counters count every test per cell; a lane forms some terms once for its VPL cells (the
// x and y parts of a box distance, of the plane height and of the in-plane coordinates), so those
// are spread over them. Per cell and test, each stage on top of the ones before whose values it
// reuses:
//   box         shared: dx 2 + dy 2 + dx^2 + dy^2 3;  per cell: dz 2 + fma 2     = 4 + 7 / VPL
//   plane       shared: x, y offsets 2 + height 3;   per cell: z offset 1 + height 2 + h^2 1
//                                                                                  = 4 + 5 / VPL
//   rectangle   shared: u, v 6;  per cell: u, v 4 + range offsets 2 + sum of squares 4
//                                                                                  = 10 + 6 / VPL
//   full test   edge AB 3 + edge AC 10 + edge BC 11 + inside 6 + sum 1             = 31
__host__ __device__ inline double distance_flops(int vpl, double box, double plane, double rect, double full) {
  const double k = vpl > 0 ? 1.0 / vpl : 1.0;
  return (4.0 + 7.0 * k) * box + (4.0 + 5.0 * k) * plane + (10.0 + 6.0 * k) * rect + 31.0 * full;
}

// ---------------------------------------------------------------------------------------------
// BVH node (64 bytes): the boxes of both children plus their references, so one 64-byte read
// yields everything a traversal step needs. A child box is stored as its centre c and half
// extent e, rounded outward so that [c - e, c + e] contains the box (an empty child has e = -inf):
//   n0 = (c0.c.x, c0.c.y, c0.c.z, c0.e.x)
//   n1 = (c0.e.y, c0.e.z, c1.c.x, c1.c.y)
//   n2 = (c1.c.z, c1.e.x, c1.e.y, c1.e.z)
//   n3 = (ref0, ref1, cnt0, cnt1) as ints: cnt == 0 -> ref is an inner node index;
//        cnt > 0 -> leaf of cnt triangles starting at triangle record ref; cnt < 0 -> empty.
struct Node {
  float4 n0, n1, n2;
  int4 n3;
};

// Squared distance from p to the box (centre c, half extent e): per axis max(|p - c| - e, 0), two
// additions and one maximum (the absolute value is an operand modifier).
__device__ __forceinline__ float box_dist2(float px, float py, float pz, float cx, float cy, float cz, float ex,
                                           float ey, float ez) {
  const float dx = fmaxf(fabsf(px - cx) - ex, 0.0f);
  const float dy = fmaxf(fabsf(py - cy) - ey, 0.0f);
  const float dz = fmaxf(fabsf(pz - cz) - ez, 0.0f);
  return dx * dx + dy * dy + dz * dz;
}

__device__ __forceinline__ void atomic_or_err(uint32_t *err, uint32_t bits) {
  if (err) atomicOr(err, bits);
}

// Orderable float <-> uint mapping for atomic min / max of floats.
__device__ __forceinline__ uint32_t float_to_ordered(float f) {
  const uint32_t u = __float_as_uint(f);
  return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}
__host__ __device__ __forceinline__ float ordered_to_float(uint32_t u) {
  const uint32_t v = (u & 0x80000000u) ? (u & 0x7fffffffu) : ~u;
#ifdef __CUDA_ARCH__
  return __uint_as_float(v);
#else
  float f;
  __builtin_memcpy(&f, &v, 4);
  return f;
#endif
}

}  // namespace sdfb
