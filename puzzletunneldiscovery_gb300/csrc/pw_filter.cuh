// pw_filter.cuh -- FP32 box and triangle tests with certified error bounds.
//
// Host and device: the device kernels use these, and host-side tests drive
// the same code against the FP64 triangle test on adversarial inputs.
#pragma once

#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>
#include <string.h>

#include "pw_math.cuh"

namespace pwf {

constexpr float U32 = 5.9604645e-08f;     // 2^-24

// FP32 value of x by truncation toward zero, computed with integer operations
// (GB300 runs FP64-to-FP32 conversions on its narrow FP64 pipe):
// |result - x| < 2^-23 |x| for 2^-126 <= |x| < 2^128; a smaller |x| gives a
// result of magnitude below 2^-126, a larger one (or a non-finite x) a finite
// result of magnitude at least 2^127.
PW_HD float f32_trunc(double x)
{
	uint64_t b;
	memcpy(&b, &x, sizeof(b));
	const uint32_t hi = (uint32_t)(b >> 32), lo = (uint32_t)b;
	constexpr uint32_t LO_EXP = 896u << 20;                  // FP64 exponent 2^-127: FP32 exponent field 0
	constexpr uint32_t HI_ABS = (1150u << 20) | 0xFFFFFu;    // largest FP64 exponent kept, 2^127
	uint32_t a = hi & 0x7FFFFFFFu;
	a = a < LO_EXP ? LO_EXP : (a > HI_ABS ? HI_ABS : a);
	const uint32_t f = (((a - LO_EXP) << 3) | (lo >> 29)) | (hi & 0x80000000u);
	float r;
	memcpy(&r, &f, sizeof(r));
	return r;
}

// Per-query FP32 transform and error bounds: five float4 per query slot in
// shared memory (80-byte stride, so lanes reading different slots hit
// different banks; lanes reading the same slot get a broadcast).
//   q[0] = (R00, R01, R02, t0)   q[1] = (R10, R11, R12, t1)   q[2] = (R20, R21, R22, t2)
//   q[3] = (er, margin, dx, W)   q[4] = (eg, 0, 0, 0)
// er:     entrywise bound on |R32 - Q|, Q the exact rotation closest to the state's (box tests)
// margin: absolute slack added to every separating-axis inequality
// dx:     per-coordinate bound on |(robot vertex - env vertex) in FP32 - the same in FP64|
// W:      bound on any coordinate magnitude (for the FP64 side's own rounding)
// eg:     a robot edge g rotates with error <= eg * |g|_1
struct QFs {
	float4 q[5];
};

// state_ulps: a further entrywise error of the state's rotation matrix against
// the reference's, in units of 2^-24, when q is not the reference's own state
// (1 for pwm::interpolate_w's frames, whose translation is the reference's).
PW_HD void make_qf(const double *q, float r1_rob, float emax_env, float del_env, QFs &o, float state_ulps = 0.f)
{
	const float x = (float)q[4], y = (float)q[5], z = (float)q[6], w = (float)q[3];
	const float tx = 2.f * x, ty = 2.f * y, tz = 2.f * z;
	const float twx = tx * w, twy = ty * w, twz = tz * w;
	const float txx = tx * x, txy = ty * x, txz = tz * x;
	const float tyy = ty * y, tyz = tz * y, tzz = tz * z;
	const float t0 = (float)q[0], t1 = (float)q[1], t2 = (float)q[2];
	o.q[0] = make_float4(1.f - (tyy + tzz), txy - twz, txz + twy, t0);
	o.q[1] = make_float4(txy + twz, 1.f - (txx + tzz), tyz - twx, t1);
	o.q[2] = make_float4(txz - twy, tyz + twx, 1.f - (txx + tyy), t2);
	const float s = x * x + y * y + z * z + w * w;
	const float dev = fabsf(1.f - s) + 8.f * U32 * s;        // |1 - |q|^2| for the FP64 quaternion
	const float epsR = (10.f * s + 4.f + state_ulps) * U32;   // |R32 - R(q64)| entrywise
	const float r1 = r1_rob;                                  // |x|_1 of any robot point (local frame)
	const float tinf = fmaxf(fmaxf(fabsf(t0), fabsf(t1)), fabsf(t2));
	const float rs = (1.f + 2.f * dev) * r1;                  // bound of |R x|_inf
	// robot vertex: rotation error, vertex rounding, three FMA roundings, t rounding, FP64 side
	const float del_r = epsR * r1 + U32 * rs + 3.f * U32 * (tinf + rs) + U32 * tinf + 1e-15f * (r1 + tinf);
	const float Wm = tinf + r1 + emax_env;
	const float er = epsR + 2.f * dev;
	const float margin = del_r + er * (3.f * r1 + 4.f * Wm) + 32.f * U32 * Wm;
	o.q[3] = make_float4(er, margin, del_r + del_env, Wm);
	o.q[4] = make_float4(epsR + 5.f * U32 * (1.f + 2.f * dev), 0.f, 0.f, 0.f);
}

// Separating-axis test of an env node box (centre A0, half-extents A1) and a
// robot node box (local centre B0, half-extents B1) placed by the slot's
// transform.  Returns a lower bound on the distance between the boxes when a
// separating axis is certified (> 0), or -1 when they may overlap.  The slack
// covers FP32 placement and arithmetic error and the distance of R32 from a
// rotation; the result is scaled down for axes whose length may exceed 1.
// EARLY: return at the first certified axis; otherwise (the kernels' form) every
// axis is evaluated without branches and the largest bound is returned: the
// same sign, and fewer instructions where most pairs of a warp overlap
// (measured: the chunk traversal 4 %, the plate's states traversal 13 % faster).
template <bool EARLY = false>
PW_HD float sat_sep32(const float4 &A0, const float4 &A1, const float4 &B0, const float4 &B1, const float4 &Q0,
                      const float4 &Q1, const float4 &Q2, const float4 &Q3)
{
	const float R00 = Q0.x, R01 = Q0.y, R02 = Q0.z, R10 = Q1.x, R11 = Q1.y, R12 = Q1.z;
	const float R20 = Q2.x, R21 = Q2.y, R22 = Q2.z;
	const float T0 = fmaf(R00, B0.x, fmaf(R01, B0.y, fmaf(R02, B0.z, Q0.w))) - A0.x;
	const float T1 = fmaf(R10, B0.x, fmaf(R11, B0.y, fmaf(R12, B0.z, Q1.w))) - A0.y;
	const float T2 = fmaf(R20, B0.x, fmaf(R21, B0.y, fmaf(R22, B0.z, Q2.w))) - A0.z;
	const float a0 = A1.x, a1 = A1.y, a2 = A1.z, b0 = B1.x, b1 = B1.y, b2 = B1.z;
	const float m = fmaf(Q3.x, (a0 + a1 + a2) + (b0 + b1 + b2), Q3.y);
	const float shrink = 1.f - 4.f * Q3.x;
	const float aR00 = fabsf(R00), aR01 = fabsf(R01), aR02 = fabsf(R02);
	const float aR10 = fabsf(R10), aR11 = fabsf(R11), aR12 = fabsf(R12);
	const float aR20 = fabsf(R20), aR21 = fabsf(R21), aR22 = fabsf(R22);
	float g, gA = -3.0e38f, gB = -3.0e38f;
	// env axes (unit length)
	g = fabsf(T0) - (a0 + fmaf(b0, aR00, fmaf(b1, aR01, fmaf(b2, aR02, m))));
	if (EARLY && g > 0.f) return g;
	gA = fmaxf(gA, g);
	g = fabsf(T1) - (a1 + fmaf(b0, aR10, fmaf(b1, aR11, fmaf(b2, aR12, m))));
	if (EARLY && g > 0.f) return g;
	gA = fmaxf(gA, g);
	g = fabsf(T2) - (a2 + fmaf(b0, aR20, fmaf(b1, aR21, fmaf(b2, aR22, m))));
	if (EARLY && g > 0.f) return g;
	gA = fmaxf(gA, g);
	// robot axes
	g = fabsf(fmaf(T0, R00, fmaf(T1, R10, T2 * R20))) - (b0 + fmaf(a0, aR00, fmaf(a1, aR10, fmaf(a2, aR20, m))));
	if (EARLY && g > 0.f) return g * shrink;
	gB = fmaxf(gB, g);
	g = fabsf(fmaf(T0, R01, fmaf(T1, R11, T2 * R21))) - (b1 + fmaf(a0, aR01, fmaf(a1, aR11, fmaf(a2, aR21, m))));
	if (EARLY && g > 0.f) return g * shrink;
	gB = fmaxf(gB, g);
	g = fabsf(fmaf(T0, R02, fmaf(T1, R12, T2 * R22))) - (b2 + fmaf(a0, aR02, fmaf(a1, aR12, fmaf(a2, aR22, m))));
	if (EARLY && g > 0.f) return g * shrink;
	gB = fmaxf(gB, g);
	// cross axes e_i x (column j of R), length at most that of the column
	g = fabsf(T2 * R10 - T1 * R20) - fmaf(a1, aR20, fmaf(a2, aR10, fmaf(b1, aR02, fmaf(b2, aR01, m))));
	if (EARLY && g > 0.f) return g * shrink;
	gB = fmaxf(gB, g);
	g = fabsf(T2 * R11 - T1 * R21) - fmaf(a1, aR21, fmaf(a2, aR11, fmaf(b0, aR02, fmaf(b2, aR00, m))));
	if (EARLY && g > 0.f) return g * shrink;
	gB = fmaxf(gB, g);
	g = fabsf(T2 * R12 - T1 * R22) - fmaf(a1, aR22, fmaf(a2, aR12, fmaf(b0, aR01, fmaf(b1, aR00, m))));
	if (EARLY && g > 0.f) return g * shrink;
	gB = fmaxf(gB, g);
	g = fabsf(T0 * R20 - T2 * R00) - fmaf(a0, aR20, fmaf(a2, aR00, fmaf(b1, aR12, fmaf(b2, aR11, m))));
	if (EARLY && g > 0.f) return g * shrink;
	gB = fmaxf(gB, g);
	g = fabsf(T0 * R21 - T2 * R01) - fmaf(a0, aR21, fmaf(a2, aR01, fmaf(b0, aR12, fmaf(b2, aR10, m))));
	if (EARLY && g > 0.f) return g * shrink;
	gB = fmaxf(gB, g);
	g = fabsf(T0 * R22 - T2 * R02) - fmaf(a0, aR22, fmaf(a2, aR02, fmaf(b0, aR11, fmaf(b1, aR10, m))));
	if (EARLY && g > 0.f) return g * shrink;
	gB = fmaxf(gB, g);
	g = fabsf(T1 * R00 - T0 * R10) - fmaf(a0, aR10, fmaf(a1, aR00, fmaf(b1, aR22, fmaf(b2, aR21, m))));
	if (EARLY && g > 0.f) return g * shrink;
	gB = fmaxf(gB, g);
	g = fabsf(T1 * R01 - T0 * R11) - fmaf(a0, aR11, fmaf(a1, aR01, fmaf(b0, aR22, fmaf(b2, aR20, m))));
	if (EARLY && g > 0.f) return g * shrink;
	gB = fmaxf(gB, g);
	g = fabsf(T1 * R02 - T0 * R12) - fmaf(a0, aR12, fmaf(a1, aR02, fmaf(b0, aR21, fmaf(b1, aR20, m))));
	if (EARLY && g > 0.f) return g * shrink;
	gB = fmaxf(gB, g);
	// a robot or cross axis counts only with a positive scale (shrink < 0: rotation error too large)
	const float sep = fmaxf(gA, gB > 0.f ? gB * shrink : -1.f);
	return sep > 0.f ? sep : -1.f;
}

PW_HD bool sat_disjoint32(const float4 &A0, const float4 &A1, const float4 &B0, const float4 &B1, const float4 &Q0,
                          const float4 &Q1, const float4 &Q2, const float4 &Q3)
{
	return sat_sep32(A0, A1, B0, B1, Q0, Q1, Q2, Q3) > 0.f;
}

// Entrywise error of a stored FP32 axis row against the orthonormal FP64 frame it
// rounds (half an ulp of an entry of magnitude <= 1, plus the FP64 frame's own
// departure from orthonormality).
constexpr float AXIS_ERR = 6.0e-8f;

// Separating-axis test of two oriented node boxes: the env node (centre A0,
// half-extents A1, axes as rows E0..E2, env frame) and the robot node (centre B0,
// half-extents B1, axes as rows G0..G2, robot frame) placed by the slot's
// transform (Q0..Q3 as in sat_sep32).  The robot box is brought into the env
// box's frame: offset T = E (R c_r + t - c_e) and rotation M = E R G^T, whose
// columns are the robot box's axes seen along the env box's axes.
//   Error model: M differs entrywise from the exact rotation E* Q G*^T (E*, G*
//   the exact orthonormal frames, Q the rotation closest to the state's) by at
//   most 3 er + 5 AXIS_ERR + 15 u (two 3-term products of matrices with unit
//   rows; u = 2^-24), doubled for safety; T differs from its exact value by the
//   robot point placement error the margin covers, seen along unit axes
//   (doubled margin), plus (AXIS_ERR + 4 u) |d|_1 (doubled) for the rounded env
//   axes and the FP32 products.  Returns a lower bound on the distance when a
//   separating axis is certified (> 0), else -1; EARLY as for sat_sep32.
template <bool EARLY = false>
PW_HD float sat_sep32_obb(const float4 &A0, const float4 &A1, const float4 &E0, const float4 &E1, const float4 &E2,
                          const float4 &B0, const float4 &B1, const float4 &G0, const float4 &G1, const float4 &G2,
                          const float4 &Q0, const float4 &Q1, const float4 &Q2, const float4 &Q3)
{
	// robot node centre in the env frame, relative to the env node centre
	const float dx = fmaf(Q0.x, B0.x, fmaf(Q0.y, B0.y, fmaf(Q0.z, B0.z, Q0.w))) - A0.x;
	const float dy = fmaf(Q1.x, B0.x, fmaf(Q1.y, B0.y, fmaf(Q1.z, B0.z, Q1.w))) - A0.y;
	const float dz = fmaf(Q2.x, B0.x, fmaf(Q2.y, B0.y, fmaf(Q2.z, B0.z, Q2.w))) - A0.z;
	const float T0 = fmaf(E0.x, dx, fmaf(E0.y, dy, E0.z * dz));
	const float T1 = fmaf(E1.x, dx, fmaf(E1.y, dy, E1.z * dz));
	const float T2 = fmaf(E2.x, dx, fmaf(E2.y, dy, E2.z * dz));
	// robot box axis j in the env frame: N_j = R g_j
	const float N00 = fmaf(Q0.x, G0.x, fmaf(Q0.y, G0.y, Q0.z * G0.z));
	const float N10 = fmaf(Q1.x, G0.x, fmaf(Q1.y, G0.y, Q1.z * G0.z));
	const float N20 = fmaf(Q2.x, G0.x, fmaf(Q2.y, G0.y, Q2.z * G0.z));
	const float N01 = fmaf(Q0.x, G1.x, fmaf(Q0.y, G1.y, Q0.z * G1.z));
	const float N11 = fmaf(Q1.x, G1.x, fmaf(Q1.y, G1.y, Q1.z * G1.z));
	const float N21 = fmaf(Q2.x, G1.x, fmaf(Q2.y, G1.y, Q2.z * G1.z));
	const float N02 = fmaf(Q0.x, G2.x, fmaf(Q0.y, G2.y, Q0.z * G2.z));
	const float N12 = fmaf(Q1.x, G2.x, fmaf(Q1.y, G2.y, Q1.z * G2.z));
	const float N22 = fmaf(Q2.x, G2.x, fmaf(Q2.y, G2.y, Q2.z * G2.z));
	// M_ij = e_i . N_j
	const float R00 = fmaf(E0.x, N00, fmaf(E0.y, N10, E0.z * N20));
	const float R01 = fmaf(E0.x, N01, fmaf(E0.y, N11, E0.z * N21));
	const float R02 = fmaf(E0.x, N02, fmaf(E0.y, N12, E0.z * N22));
	const float R10 = fmaf(E1.x, N00, fmaf(E1.y, N10, E1.z * N20));
	const float R11 = fmaf(E1.x, N01, fmaf(E1.y, N11, E1.z * N21));
	const float R12 = fmaf(E1.x, N02, fmaf(E1.y, N12, E1.z * N22));
	const float R20 = fmaf(E2.x, N00, fmaf(E2.y, N10, E2.z * N20));
	const float R21 = fmaf(E2.x, N01, fmaf(E2.y, N11, E2.z * N21));
	const float R22 = fmaf(E2.x, N02, fmaf(E2.y, N12, E2.z * N22));
	const float a0 = A1.x, a1 = A1.y, a2 = A1.z, b0 = B1.x, b1 = B1.y, b2 = B1.z;
	const float er = fmaf(6.f, Q3.x, 2.f * (5.f * AXIS_ERR + 15.f * U32));
	const float eT = 2.f * (AXIS_ERR + 4.f * U32) * (fabsf(dx) + fabsf(dy) + fabsf(dz));
	const float m = fmaf(er, (a0 + a1 + a2) + (b0 + b1 + b2), fmaf(2.f, Q3.y, eT));
	const float shrink = 1.f - 4.f * er;
	const float aR00 = fabsf(R00), aR01 = fabsf(R01), aR02 = fabsf(R02);
	const float aR10 = fabsf(R10), aR11 = fabsf(R11), aR12 = fabsf(R12);
	const float aR20 = fabsf(R20), aR21 = fabsf(R21), aR22 = fabsf(R22);
	float g, gA = -3.0e38f, gB = -3.0e38f;
	// env box axes (unit length)
	g = fabsf(T0) - (a0 + fmaf(b0, aR00, fmaf(b1, aR01, fmaf(b2, aR02, m))));
	if (EARLY && g > 0.f) return g;
	gA = fmaxf(gA, g);
	g = fabsf(T1) - (a1 + fmaf(b0, aR10, fmaf(b1, aR11, fmaf(b2, aR12, m))));
	if (EARLY && g > 0.f) return g;
	gA = fmaxf(gA, g);
	g = fabsf(T2) - (a2 + fmaf(b0, aR20, fmaf(b1, aR21, fmaf(b2, aR22, m))));
	if (EARLY && g > 0.f) return g;
	gA = fmaxf(gA, g);
	// robot box axes
	g = fabsf(fmaf(T0, R00, fmaf(T1, R10, T2 * R20))) - (b0 + fmaf(a0, aR00, fmaf(a1, aR10, fmaf(a2, aR20, m))));
	if (EARLY && g > 0.f) return g * shrink;
	gB = fmaxf(gB, g);
	g = fabsf(fmaf(T0, R01, fmaf(T1, R11, T2 * R21))) - (b1 + fmaf(a0, aR01, fmaf(a1, aR11, fmaf(a2, aR21, m))));
	if (EARLY && g > 0.f) return g * shrink;
	gB = fmaxf(gB, g);
	g = fabsf(fmaf(T0, R02, fmaf(T1, R12, T2 * R22))) - (b2 + fmaf(a0, aR02, fmaf(a1, aR12, fmaf(a2, aR22, m))));
	if (EARLY && g > 0.f) return g * shrink;
	gB = fmaxf(gB, g);
	// cross axes e_i x (column j of M)
	g = fabsf(T2 * R10 - T1 * R20) - fmaf(a1, aR20, fmaf(a2, aR10, fmaf(b1, aR02, fmaf(b2, aR01, m))));
	if (EARLY && g > 0.f) return g * shrink;
	gB = fmaxf(gB, g);
	g = fabsf(T2 * R11 - T1 * R21) - fmaf(a1, aR21, fmaf(a2, aR11, fmaf(b0, aR02, fmaf(b2, aR00, m))));
	if (EARLY && g > 0.f) return g * shrink;
	gB = fmaxf(gB, g);
	g = fabsf(T2 * R12 - T1 * R22) - fmaf(a1, aR22, fmaf(a2, aR12, fmaf(b0, aR01, fmaf(b1, aR00, m))));
	if (EARLY && g > 0.f) return g * shrink;
	gB = fmaxf(gB, g);
	g = fabsf(T0 * R20 - T2 * R00) - fmaf(a0, aR20, fmaf(a2, aR00, fmaf(b1, aR12, fmaf(b2, aR11, m))));
	if (EARLY && g > 0.f) return g * shrink;
	gB = fmaxf(gB, g);
	g = fabsf(T0 * R21 - T2 * R01) - fmaf(a0, aR21, fmaf(a2, aR01, fmaf(b0, aR12, fmaf(b2, aR10, m))));
	if (EARLY && g > 0.f) return g * shrink;
	gB = fmaxf(gB, g);
	g = fabsf(T0 * R22 - T2 * R02) - fmaf(a0, aR22, fmaf(a2, aR02, fmaf(b0, aR11, fmaf(b1, aR10, m))));
	if (EARLY && g > 0.f) return g * shrink;
	gB = fmaxf(gB, g);
	g = fabsf(T1 * R00 - T0 * R10) - fmaf(a0, aR10, fmaf(a1, aR00, fmaf(b1, aR22, fmaf(b2, aR21, m))));
	if (EARLY && g > 0.f) return g * shrink;
	gB = fmaxf(gB, g);
	g = fabsf(T1 * R01 - T0 * R11) - fmaf(a0, aR11, fmaf(a1, aR01, fmaf(b0, aR22, fmaf(b2, aR20, m))));
	if (EARLY && g > 0.f) return g * shrink;
	gB = fmaxf(gB, g);
	g = fabsf(T1 * R02 - T0 * R12) - fmaf(a0, aR12, fmaf(a1, aR02, fmaf(b0, aR21, fmaf(b1, aR20, m))));
	if (EARLY && g > 0.f) return g * shrink;
	gB = fmaxf(gB, g);
	// a robot or cross axis counts only with a positive scale (shrink < 0: rotation error too large)
	const float sep = fmaxf(gA, gB > 0.f ? gB * shrink : -1.f);
	return sep > 0.f ? sep : -1.f;
}

PW_HD float3 f3(float4 a) { return make_float3(a.x, a.y, a.z); }
PW_HD float3 f3add(float3 a, float3 b) { return make_float3(a.x + b.x, a.y + b.y, a.z + b.z); }
PW_HD float3 f3sub(float3 a, float3 b) { return make_float3(a.x - b.x, a.y - b.y, a.z - b.z); }
PW_HD float3 f3neg(float3 a) { return make_float3(-a.x, -a.y, -a.z); }
PW_HD float3 f3cross(float3 a, float3 b)
{
	return make_float3(fmaf(a.y, b.z, -a.z * b.y), fmaf(a.z, b.x, -a.x * b.z), fmaf(a.x, b.y, -a.y * b.x));
}
PW_HD float f3dot(float3 a, float3 b) { return fmaf(a.x, b.x, fmaf(a.y, b.y, a.z * b.z)); }
PW_HD float f3inf(float3 a) { return fmaxf(fmaxf(fabsf(a.x), fabsf(a.y)), fabsf(a.z)); }
PW_HD float f3l1(float3 a) { return fabsf(a.x) + fabsf(a.y) + fabsf(a.z); }
PW_HD float f3get(float3 a, int i) { return i == 0 ? a.x : (i == 1 ? a.y : a.z); }

// Signed distances of three points (given relative to the plane's first vertex,
// w[k] with per-coordinate error ew[k]) to the plane with normal N = e1 x e2,
// and a bound b[k] on |FP32 value - FP64 value (Moeller's formula)|.
struct PlaneRes {
	float3 N;
	float etaN, NL1;
	float d[3], b[3];
};

PW_HD void plane_bounds(float3 e1, float3 e2, float ee1, float ee2, const float3 *w,
                                             const float *ew, float M, PlaneRes &r)
{
	r.N = f3cross(e1, e2);
	const float A1 = f3inf(e1), A2 = f3inf(e2);
	r.etaN = 2.f * (A1 * ee2 + ee1 * A2 + ee1 * ee2) + 3.f * U32 * A1 * A2;
	const float NL1 = f3l1(r.N) + 3.f * r.etaN;
	r.NL1 = NL1;
	const float b64 = 4e-15f * (NL1 + 4.f * A1 * A2) * M;
#pragma unroll
	for (int k = 0; k < 3; k++) {
		const float Wi = f3inf(w[k]), W1 = f3l1(w[k]);
		r.d[k] = f3dot(r.N, w[k]);
		r.b[k] = 2.f * (NL1 * ew[k] + r.etaN * (W1 + 3.f * ew[k]) + 3.f * U32 * NL1 * Wi + b64);
	}
}

// -1 / +1 certified sign, 0 uncertain.
PW_HD int csign(float d, float b) { return d > b ? 1 : (d < -b ? -1 : 0); }

// Lone vertex from certified nonzero signs (mirrors the FP64 dispatch).
PW_HD int lone3(const int *s)
{
	if (s[0] * s[1] > 0) return 2;
	if (s[0] * s[2] > 0) return 1;
	return 0;
}

// a[i] for a runtime i in {0, 1, 2}, by selects: the arrays stay in registers
// (indexing them with a runtime value would move them to local memory).
PW_HD float sel3(const float *a, int i) { return i == 0 ? a[0] : (i == 1 ? a[1] : a[2]); }

// Interval on the projection axis: endpoints p_l + (p_o - p_l) d_l / (d_l - d_o)
// with p relative to a common origin.  ea[k]: error of p[k]; ei[k]: the part of
// it that does not cancel in differences.  Returns the endpoints and a bound.
PW_HD void interval_bounds(const float *p, const float *ea, const float *ei, const float *d,
                                                const float *b, int lone, float *lo, float *hi, float *err)
{
	const int o1 = lone == 0 ? 1 : 0;
	const int o2 = lone == 2 ? 1 : 2;
	const float pl = sel3(p, lone), eal = sel3(ea, lone), eil = sel3(ei, lone);
	const float dl = sel3(d, lone), bl = sel3(b, lone);
	float e[2], E = 0.f;
#pragma unroll
	for (int k = 0; k < 2; k++) {
		const int o = k == 0 ? o1 : o2;
		const float d_o = sel3(d, o), b_o = sel3(b, o), p_o = sel3(p, o), ei_o = sel3(ei, o);
		const float den = fabsf(dl) + fabsf(d_o);
		const float bb = bl + b_o;
		const float r = dl / (dl - d_o);
		const float dr = bb / fmaxf(den - bb, 1e-37f) + 3.f * U32;
		const float pd = p_o - pl;
		e[k] = fmaf(pd, r, pl);
		const float epd = ei_o + eil + U32 * fabsf(pd);
		const float ek = eal + epd + fabsf(pd) * dr + U32 * (fabsf(pl) + 2.f * fabsf(pd));
		E = fmaxf(E, ek);
	}
	*lo = fminf(e[0], e[1]);
	*hi = fmaxf(e[0], e[1]);
	*err = E;
}

// Lower bound on the distance between a triangle and the points of a plane
// test whose signs are all certified equal: min (|d| - b) / |N|_1.
PW_HD float plane_gap(const PlaneRes &r)
{
	float g = fabsf(r.d[0]) - r.b[0];
	g = fminf(g, fabsf(r.d[1]) - r.b[1]);
	g = fminf(g, fabsf(r.d[2]) - r.b[2]);
	return fmaxf(g, 0.f) / r.NL1;
}

// FP32 Moeller filter of env triangle (V0, edges e1, e2) against robot triangle
// (local vertex x0, local edges g1, g2) placed by the slot's transform.
// 0 = certified separate, 1 = certified intersecting, 2 = uncertain.
// *gap: a lower bound on the distance between the triangles (0 when unknown).
PW_HD int tri_filter(float3 V0, float3 e1, float3 e2, float3 x0, float3 g1, float3 g2, const float4 &Q0,
                     const float4 &Q1, const float4 &Q2, const float4 &Q3, float eg, float *gap)
{
	*gap = 0.f;
	const float dx = Q3.z, M = Q3.w;
	const float3 U0 = make_float3(fmaf(Q0.x, x0.x, fmaf(Q0.y, x0.y, fmaf(Q0.z, x0.z, Q0.w))),
	                              fmaf(Q1.x, x0.x, fmaf(Q1.y, x0.y, fmaf(Q1.z, x0.z, Q1.w))),
	                              fmaf(Q2.x, x0.x, fmaf(Q2.y, x0.y, fmaf(Q2.z, x0.z, Q2.w))));
	const float3 f1 = make_float3(fmaf(Q0.x, g1.x, fmaf(Q0.y, g1.y, Q0.z * g1.z)),
	                              fmaf(Q1.x, g1.x, fmaf(Q1.y, g1.y, Q1.z * g1.z)),
	                              fmaf(Q2.x, g1.x, fmaf(Q2.y, g1.y, Q2.z * g1.z)));
	const float3 f2 = make_float3(fmaf(Q0.x, g2.x, fmaf(Q0.y, g2.y, Q0.z * g2.z)),
	                              fmaf(Q1.x, g2.x, fmaf(Q1.y, g2.y, Q1.z * g2.z)),
	                              fmaf(Q2.x, g2.x, fmaf(Q2.y, g2.y, Q2.z * g2.z)));
	const float G1 = eg * f3l1(g1) + 1e-15f * M, G2 = eg * f3l1(g2) + 1e-15f * M;   // errors of f1, f2
	const float A1 = f3inf(e1), A2 = f3inf(e2);
	const float3 w0 = f3sub(U0, V0);                       // U0 - V0
	const float ew0 = dx + U32 * f3inf(w0);
	// robot vertices relative to V0: du = N1 . (U_k - V0)
	float3 w[3];
	float ew[3], eiu[3];
	w[0] = w0;
	w[1] = f3add(w0, f1);
	w[2] = f3add(w0, f2);
	ew[0] = ew0;
	ew[1] = ew0 + G1 + U32 * f3inf(w[1]);
	ew[2] = ew0 + G2 + U32 * f3inf(w[2]);
	PlaneRes pv;
	plane_bounds(e1, e2, U32 * A1, U32 * A2, w, ew, M, pv);
	int su[3];
#pragma unroll
	for (int k = 0; k < 3; k++) su[k] = csign(pv.d[k], pv.b[k]);
	if (su[0] == 0 || su[1] == 0 || su[2] == 0)
		return 2;
	if (su[0] == su[1] && su[0] == su[2]) {
		*gap = plane_gap(pv);
		return 0;
	}
	// env vertices relative to U0: dv = N2 . (V_i - U0)
	float3 v[3];
	float evv[3];
	v[0] = f3neg(w0);
	v[1] = f3add(v[0], e1);
	v[2] = f3add(v[0], e2);
	evv[0] = ew0;
	evv[1] = ew0 + U32 * A1 + U32 * f3inf(v[1]);
	evv[2] = ew0 + U32 * A2 + U32 * f3inf(v[2]);
	PlaneRes pu;
	plane_bounds(f1, f2, G1, G2, v, evv, M, pu);
	int sv[3];
#pragma unroll
	for (int k = 0; k < 3; k++) sv[k] = csign(pu.d[k], pu.b[k]);
	if (sv[0] == 0 || sv[1] == 0 || sv[2] == 0)
		return 2;
	if (sv[0] == sv[1] && sv[0] == sv[2]) {
		*gap = plane_gap(pu);
		return 0;
	}
	// direction of the intersection line and the FP64 axis choice
	const float3 Dl = f3cross(pv.N, pu.N);
	const float n1 = f3inf(pv.N), n2 = f3inf(pu.N);
	const float etaD = 2.f * (2.f * (n1 * pu.etaN + pv.etaN * n2 + pv.etaN * pu.etaN) + 3.f * U32 * n1 * n2 +
	                          3e-14f * n1 * n2);
	const float a0 = fabsf(Dl.x), a1 = fabsf(Dl.y), a2 = fabsf(Dl.z);
	int ax = 0;
	float mx = a0;
	if (a1 > mx) { mx = a1; ax = 1; }
	if (a2 > mx) { mx = a2; ax = 2; }
	const float o_a = ax == 0 ? a1 : a0;
	const float o_b = ax == 2 ? a1 : a2;
	if (mx - o_a <= 2.f * etaD || mx - o_b <= 2.f * etaD)
		return 2;
	// projections relative to V0 on the chosen axis
	const float pvv[3] = { 0.f, f3get(e1, ax), f3get(e2, ax) };
	const float eav[3] = { 0.f, U32 * A1, U32 * A2 };
	const float puu[3] = { f3get(w[0], ax), f3get(w[1], ax), f3get(w[2], ax) };
	const float eau[3] = { ew[0], ew[1], ew[2] };
	eiu[0] = U32 * fabsf(puu[0]);
	eiu[1] = G1 + U32 * fabsf(puu[1]);
	eiu[2] = G2 + U32 * fabsf(puu[2]);
	float vlo, vhi, verr, ulo, uhi, uerr;
	interval_bounds(pvv, eav, eav, pu.d, pu.b, lone3(sv), &vlo, &vhi, &verr);
	interval_bounds(puu, eau, eiu, pv.d, pv.b, lone3(su), &ulo, &uhi, &uerr);
	const float B = 2.f * (verr + uerr + 1e-14f * M);
	const float s1 = ulo - vhi, s2 = vlo - uhi;
	if (s1 > B || s2 > B)
		return 0;
	if (s1 < -B && s2 < -B)
		return 1;
	return 2;
}


// ---------------------------------------------------------------- isDisentangled in FP32
//
// UnitWorld::isDisentangled (unit_world.cc:249-264, CDModel::collideBB,
// cdmodel.cc:180-197): the robot's bounding box (centre rc, half-extents rh,
// robot frame) placed by the state against the environment's box (ec, eh)
// placed by the perturbation (Re, te); pwm::boxes_disjoint computes it in FP64.
// Here the same separating-axis test runs in FP32 with one error bound e for
// all 15 axes:
//   1  (disjoint) if some axis has  |tl| - (ra + rb) >  e,
//   0  (overlap)  if every axis has |tl| - (ra + rb) < -e,
//   -1 otherwise: the FP64 test decides.
// e bounds |g32 - g| + |g64 - g| for every axis value g (exact), g32 (this
// code), g64 (the FP64 test).  R is the rotation formula on the state's raw
// quaternion (as the FP64 test and Eigen's toRotationMatrix apply it, unit or
// not), so its entries are bounded by K = max(1, 2 |q|^2).  The state's seven
// components are truncated to FP32 with integer operations (f32_trunc, relative
// error below 2u; the FP64 pipe is GB300's narrowest), so the computed |q|^2 is
// at least |q|^2 (1 - 7u) and K carries a factor 1 + 16u.  With u = 2^-24, the
// entrywise error of R is at most 10 K u (from the truncated components and the
// roundings of the quadratic entries: at most 7 K u on the diagonal, 3 K u off
// it), of d = R rc + t - ce at most (10 K + 7) u (|rc|_1 +
// |t|_inf + |ce|_inf + |d|_inf; t truncated, 2u), of
// T = Re^T d at most 2 eps_d + 4u |d|_1, of Re^T R at most (20 K + 5) u (each
// operation rounded once or, fused, fewer times); the axis values are sums of at most six such
// terms weighted by |T|_inf <= |d|_1, the extents and K, so
// e = 1100u K (|rc|_1 + |t|_inf + |ce|_inf + 2 |d|_1 + sum eh + sum rh) covers
// the FP32 side with a factor above 1.5 and the FP64 side (the same sums at
// 2^-53) many times over.  tests/harness/disentangled_bounds.cc checks it
// against pwm::boxes_disjoint near the boundary (slack scales e; the kernels
// use 1, the harness also runs 0 to show that the check has teeth).
struct DisBoxes32 {
	float rc[3], rh[3];    // robot box (robot frame)
	float Re[9];           // perturbation rotation (row-major)
	float ce[3];           // env box centre placed by the perturbation, Re ec + te (FP64, rounded)
	float eh[3];           // env box half-extents
	float ce_abs;          // |ce|_inf, rounded up
};

// Two FP32 lanes computed together: packed f32x2 instructions on the device
// (each lane rounded as the scalar instruction rounds it, two lanes per
// instruction), scalar code on the host.  The box test below runs on either a
// float or an F2, so one state or two share the same arithmetic.
struct F2 {
	float x, y;
};
#if defined(__CUDA_ARCH__)
__device__ __forceinline__ unsigned long long f2pack(F2 a)
{
	unsigned long long r;
	asm("mov.b64 %0, {%1, %2};" : "=l"(r) : "f"(a.x), "f"(a.y));
	return r;
}
__device__ __forceinline__ F2 f2unpack(unsigned long long v)
{
	F2 r;
	asm("mov.b64 {%0, %1}, %2;" : "=f"(r.x), "=f"(r.y) : "l"(v));
	return r;
}
__device__ __forceinline__ F2 vadd(F2 a, F2 b)
{
	unsigned long long r;
	asm("add.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(f2pack(a)), "l"(f2pack(b)));
	return f2unpack(r);
}
__device__ __forceinline__ F2 vsub(F2 a, F2 b)
{
	unsigned long long r;
	asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(f2pack(a)), "l"(f2pack(b)));
	return f2unpack(r);
}
__device__ __forceinline__ F2 vmul(F2 a, F2 b)
{
	unsigned long long r;
	asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(f2pack(a)), "l"(f2pack(b)));
	return f2unpack(r);
}
__device__ __forceinline__ F2 vfma(F2 a, F2 b, F2 c)
{
	unsigned long long r;
	asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(r) : "l"(f2pack(a)), "l"(f2pack(b)), "l"(f2pack(c)));
	return f2unpack(r);
}
#else
inline F2 vadd(F2 a, F2 b) { return { a.x + b.x, a.y + b.y }; }
inline F2 vsub(F2 a, F2 b) { return { a.x - b.x, a.y - b.y }; }
inline F2 vmul(F2 a, F2 b) { return { a.x * b.x, a.y * b.y }; }
inline F2 vfma(F2 a, F2 b, F2 c) { return { fmaf(a.x, b.x, c.x), fmaf(a.y, b.y, c.y) }; }
#endif
PW_HD F2 vabs(F2 a) { return { fabsf(a.x), fabsf(a.y) }; }
PW_HD F2 vmax(F2 a, F2 b) { return { fmaxf(a.x, b.x), fmaxf(a.y, b.y) }; }
PW_HD float vadd(float a, float b) { return a + b; }
PW_HD float vsub(float a, float b) { return a - b; }
PW_HD float vmul(float a, float b) { return a * b; }
PW_HD float vfma(float a, float b, float c) { return fmaf(a, b, c); }
PW_HD float vabs(float a) { return fabsf(a); }
PW_HD float vmax(float a, float b) { return fmaxf(a, b); }
template <typename V> PW_HD V vset(float a);
template <> PW_HD float vset<float>(float a) { return a; }
template <> PW_HD F2 vset<F2>(float a) { return { a, a }; }

// The 15 axis values of the box test for the state (w, x, y, z, t): the largest
// (g), the error bound e and |q|^2 (n2), lane by lane.  ROT = false when the
// perturbation rotation Re is exactly the identity: then Re^T d = d and
// Re^T R = R exactly (products by 1 and sums with zeros), so both are taken as
// they are.
template <bool ROT, typename V>
PW_HD void box_axes(V w, V x, V y, V z, const V t[3], const DisBoxes32 &B, float slack, V &g, V &e, V &n2)
{
	const V one = vset<V>(1.f), two = vset<V>(2.f), mtwo = vset<V>(-2.f);
	n2 = vfma(z, z, vfma(y, y, vfma(x, x, vmul(w, w))));
	const V K = vmul(vmax(one, vmul(two, n2)), vset<V>(1.f + 16.f * U32));
	const V nw = vsub(vset<V>(0.f), w);
	V R[9];
	R[0] = vfma(mtwo, vfma(y, y, vmul(z, z)), one);
	R[1] = vmul(two, vfma(x, y, vmul(nw, z)));
	R[2] = vmul(two, vfma(x, z, vmul(w, y)));
	R[3] = vmul(two, vfma(x, y, vmul(w, z)));
	R[4] = vfma(mtwo, vfma(x, x, vmul(z, z)), one);
	R[5] = vmul(two, vfma(y, z, vmul(nw, x)));
	R[6] = vmul(two, vfma(x, z, vmul(nw, y)));
	R[7] = vmul(two, vfma(y, z, vmul(w, x)));
	R[8] = vfma(mtwo, vfma(x, x, vmul(y, y)), one);
	V d[3];
	for (int k = 0; k < 3; k++)
		d[k] = vsub(vadd(vfma(R[3 * k + 2], vset<V>(B.rc[2]),
		                      vfma(R[3 * k + 1], vset<V>(B.rc[1]), vmul(R[3 * k], vset<V>(B.rc[0])))),
		                 t[k]),
		            vset<V>(B.ce[k]));
	V T[3], Rr[9], AR[9];
	for (int i = 0; i < 3; i++) {
		T[i] = ROT ? vfma(vset<V>(B.Re[6 + i]), d[2], vfma(vset<V>(B.Re[3 + i]), d[1], vmul(vset<V>(B.Re[i]), d[0])))
		           : d[i];
		for (int j = 0; j < 3; j++) {
			Rr[3 * i + j] = ROT ? vfma(vset<V>(B.Re[6 + i]), R[6 + j],
			                           vfma(vset<V>(B.Re[3 + i]), R[3 + j], vmul(vset<V>(B.Re[i]), R[j])))
			                    : R[3 * i + j];
			AR[3 * i + j] = vabs(Rr[3 * i + j]);
		}
	}
	const V d1 = vadd(vadd(vabs(d[0]), vabs(d[1])), vabs(d[2]));
	const V tinf = vmax(vmax(vabs(t[0]), vabs(t[1])), vabs(t[2]));
	const float fixed = ((fabsf(B.rc[0]) + fabsf(B.rc[1])) + fabsf(B.rc[2])) + B.ce_abs +
	                    ((B.eh[0] + B.eh[1]) + B.eh[2]) + ((B.rh[0] + B.rh[1]) + B.rh[2]);
	const V scale = vadd(vfma(two, d1, tinf), vset<V>(fixed));
	e = vmul(vset<V>(slack * 1100.f * U32), vmul(K, scale));
	g = vset<V>(-3.0e38f);
	for (int i = 0; i < 3; i++)
		g = vmax(g, vsub(vabs(T[i]), vadd(vset<V>(B.eh[i]),
		                                  vfma(vset<V>(B.rh[2]), AR[3 * i + 2],
		                                       vfma(vset<V>(B.rh[1]), AR[3 * i + 1], vmul(vset<V>(B.rh[0]), AR[3 * i]))))));
	for (int j = 0; j < 3; j++) {
		const V tl = vfma(T[2], Rr[6 + j], vfma(T[1], Rr[3 + j], vmul(T[0], Rr[j])));
		const V ra = vfma(vset<V>(B.eh[2]), AR[6 + j], vfma(vset<V>(B.eh[1]), AR[3 + j], vmul(vset<V>(B.eh[0]), AR[j])));
		g = vmax(g, vsub(vabs(tl), vadd(ra, vset<V>(B.rh[j]))));
	}
	for (int i = 0; i < 3; i++) {
		const int i1 = (i + 1) % 3, i2 = (i + 2) % 3;
		for (int j = 0; j < 3; j++) {
			const int j1 = (j + 1) % 3, j2 = (j + 2) % 3;
			const V tl = vfma(T[i2], Rr[3 * i1 + j], vmul(vsub(vset<V>(0.f), T[i1]), Rr[3 * i2 + j]));
			const V ra = vfma(vset<V>(B.eh[i1]), AR[3 * i2 + j], vmul(vset<V>(B.eh[i2]), AR[3 * i1 + j]));
			const V rb = vfma(vset<V>(B.rh[j1]), AR[3 * i + j2], vmul(vset<V>(B.rh[j2]), AR[3 * i + j1]));
			g = vmax(g, vsub(vabs(tl), vadd(ra, rb)));
		}
	}
}

// A lane's verdict from box_axes: 1 (disjoint) when g > e, 0 (overlap) when
// g < -e, -1 (the FP64 test decides) otherwise or when |q|^2 or e is not finite
// and below 1e30 (then every axis value is finite).
PW_HD int box_verdict(float g, float e, float n2)
{
	if (!(n2 < 1.0e30f) || !(e < 1.0e30f))
		return -1;
	return g > e ? 1 : (g < -e ? 0 : -1);
}

template <bool ROT>
PW_HD int boxes_disjoint32(const double *q, const DisBoxes32 &B, float slack = 1.f)
{
	const float t[3] = { f32_trunc(q[0]), f32_trunc(q[1]), f32_trunc(q[2]) };
	float g, e, n2;
	box_axes<ROT, float>(f32_trunc(q[3]), f32_trunc(q[4]), f32_trunc(q[5]), f32_trunc(q[6]), t, B, slack, g, e, n2);
	return box_verdict(g, e, n2);
}

// The same test for two states at once (packed arithmetic on the device).
template <bool ROT>
PW_HD void boxes_disjoint32x2(const double *qa, const double *qb, const DisBoxes32 &B, int &va, int &vb,
                              float slack = 1.f)
{
	F2 t[3];
	for (int c = 0; c < 3; c++)
		t[c] = { f32_trunc(qa[c]), f32_trunc(qb[c]) };
	F2 g, e, n2;
	box_axes<ROT, F2>({ f32_trunc(qa[3]), f32_trunc(qb[3]) }, { f32_trunc(qa[4]), f32_trunc(qb[4]) },
	                  { f32_trunc(qa[5]), f32_trunc(qb[5]) }, { f32_trunc(qa[6]), f32_trunc(qb[6]) }, t, B, slack, g, e,
	                  n2);
	va = box_verdict(g.x, e.x, n2.x);
	vb = box_verdict(g.y, e.y, n2.y);
}

} // namespace pwf
