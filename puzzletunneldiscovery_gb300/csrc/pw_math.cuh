// pw_math.cuh -- deterministic FP64 math shared by host and device code.
//
// Every FP64 operation here is separately rounded: on the device through the
// __d*_rn intrinsics (which the compiler never fuses into FMAs), on the host
// through plain operators compiled with -ffp-contract=off.  Host and device
// therefore produce bit-identical states, transforms and triangle verdicts.
//
// Restated behaviour:
//   state -> transform           lib/osr/osr_state.cc:16-25 (raw quaternion)
//   interpolate (lerp + slerp)   lib/osr/osr_state.cc:27-44
//   decompose / compose          lib/osr/osr_state.cc:85-119
//   distance                     lib/osr/osr_state.cc:130-154
//   triangle-triangle test       Moeller, JGT 2(2) 1997 (lib/tritri/Moller97d.cc:220,579)
// sin / acos / atan2 are this file's own: Taylor series after complement and
// half-angle argument reduction, accurate to a few ulp on the ranges used.
#pragma once

#include <math.h>
#include <stdint.h>
#include <string.h>

#if defined(__CUDACC__)
#define PW_HD __host__ __device__ __forceinline__
#else
#define PW_HD inline
#endif

namespace pwm {

#if defined(__CUDA_ARCH__)
PW_HD double add(double a, double b) { return __dadd_rn(a, b); }
PW_HD double sub(double a, double b) { return __dsub_rn(a, b); }
PW_HD double mul(double a, double b) { return __dmul_rn(a, b); }
PW_HD double dvd(double a, double b) { return __ddiv_rn(a, b); }
PW_HD double rt(double a) { return __dsqrt_rn(a); }
PW_HD double fmad(double a, double b, double c) { return __fma_rn(a, b, c); }
#else
PW_HD double add(double a, double b) { return a + b; }
PW_HD double sub(double a, double b) { return a - b; }
PW_HD double mul(double a, double b) { return a * b; }
PW_HD double dvd(double a, double b) { return a / b; }
PW_HD double rt(double a) { return sqrt(a); }
PW_HD double fmad(double a, double b, double c) { return fma(a, b, c); }
#endif
PW_HD double dabs(double a) { return a >= 0.0 ? a : -a; }

constexpr double PIO2_HI = 1.5707963267948965579989817342720925807952880859375;
constexpr double PIO2_LO = 6.123233995736766035868820147291818e-17;
constexpr double PIO4_HI = 0.78539816339744827899949086713604629039764404296875;
constexpr double PIO4_LO = 3.061616997868383017934410073645909e-17;
constexpr double TAN_PI_8 = 0.41421356237309503;
constexpr double SLERP_ONE = 1.0 - 2.220446049250313080847e-16;

PW_HD double sin_kernel(double x)
{
	const double z = mul(x, x);
	double p = 2.8114572543455207632e-15;
	p = sub(mul(p, z), 7.6471637318198164759e-13);
	p = add(mul(p, z), 1.6059043836821614599e-10);
	p = sub(mul(p, z), 2.5052108385441718775e-08);
	p = add(mul(p, z), 2.7557319223985890653e-06);
	p = sub(mul(p, z), 1.9841269841269841270e-04);
	p = add(mul(p, z), 8.3333333333333333333e-03);
	p = sub(mul(p, z), 1.6666666666666666667e-01);
	return add(x, mul(x, mul(z, p)));
}

PW_HD double cos_kernel(double y)
{
	const double z = mul(y, y);
	double p = -1.5619206968586225271e-16;
	p = add(mul(p, z), 4.7794773323873852974e-14);
	p = sub(mul(p, z), 1.1470745597729724714e-11);
	p = add(mul(p, z), 2.0876756987868098979e-09);
	p = sub(mul(p, z), 2.7557319223985890653e-07);
	p = add(mul(p, z), 2.4801587301587301587e-05);
	p = sub(mul(p, z), 1.3888888888888888889e-03);
	p = add(mul(p, z), 4.1666666666666666667e-02);
	p = sub(mul(p, z), 5.0000000000000000000e-01);
	return add(1.0, mul(z, p));
}

// sin(x) for x in [-pi/4, pi/2 + small].
PW_HD double sin_q(double x)
{
	if (x <= PIO4_HI)
		return sin_kernel(x);
	return cos_kernel(add(sub(PIO2_HI, x), PIO2_LO));
}

// The same polynomials evaluated with fused multiply-adds (half the FP64
// instructions), for frames that only feed the certified FP32 filters: not the
// reference's rounding, within a few units of 2^-53 of sin_q on its range.
PW_HD double sin_kernel_f(double x)
{
	const double z = mul(x, x);
	double p = 2.8114572543455207632e-15;
	p = fmad(p, z, -7.6471637318198164759e-13);
	p = fmad(p, z, 1.6059043836821614599e-10);
	p = fmad(p, z, -2.5052108385441718775e-08);
	p = fmad(p, z, 2.7557319223985890653e-06);
	p = fmad(p, z, -1.9841269841269841270e-04);
	p = fmad(p, z, 8.3333333333333333333e-03);
	p = fmad(p, z, -1.6666666666666666667e-01);
	return fmad(mul(x, z), p, x);
}

PW_HD double cos_kernel_f(double y)
{
	const double z = mul(y, y);
	double p = -1.5619206968586225271e-16;
	p = fmad(p, z, 4.7794773323873852974e-14);
	p = fmad(p, z, -1.1470745597729724714e-11);
	p = fmad(p, z, 2.0876756987868098979e-09);
	p = fmad(p, z, -2.7557319223985890653e-07);
	p = fmad(p, z, 2.4801587301587301587e-05);
	p = fmad(p, z, -1.3888888888888888889e-03);
	p = fmad(p, z, 4.1666666666666666667e-02);
	p = fmad(p, z, -5.0000000000000000000e-01);
	return fmad(z, p, 1.0);
}

PW_HD double sin_qf(double x)
{
	if (x <= PIO4_HI)
		return sin_kernel_f(x);
	return cos_kernel_f(add(sub(PIO2_HI, x), PIO2_LO));
}

// atan(z) for z in [0, 1].
PW_HD double atan01(double z)
{
	bool shifted = false;
	if (z > TAN_PI_8) {
		z = dvd(sub(z, 1.0), add(z, 1.0));
		shifted = true;
	}
	const double w = dvd(z, add(1.0, rt(add(1.0, mul(z, z)))));
	const double s = mul(w, w);
	double p = 0.043478260869565216;
	p = sub(mul(p, s), 0.047619047619047616);
	p = add(mul(p, s), 0.05263157894736842);
	p = sub(mul(p, s), 0.058823529411764705);
	p = add(mul(p, s), 0.06666666666666667);
	p = sub(mul(p, s), 0.07692307692307693);
	p = add(mul(p, s), 0.09090909090909091);
	p = sub(mul(p, s), 0.1111111111111111);
	p = add(mul(p, s), 0.14285714285714285);
	p = sub(mul(p, s), 0.2);
	p = add(mul(p, s), 0.3333333333333333);
	const double a = sub(w, mul(w, mul(s, p)));
	double r = mul(2.0, a);
	if (shifted)
		r = add(PIO4_HI, add(r, PIO4_LO));
	return r;
}

// atan2(y, x) for y >= 0, x >= 0.
PW_HD double atan2q(double y, double x)
{
	if (y == 0.0)
		return 0.0;
	if (y <= x)
		return atan01(dvd(y, x));
	return add(sub(PIO2_HI, atan01(dvd(x, y))), PIO2_LO);
}

// acos(a) for a in [0, 1].
PW_HD double acos01(double a)
{
	return mul(2.0, atan2q(rt(sub(1.0, a)), rt(add(1.0, a))));
}

// ---------------------------------------------------------------- states

// Quaternions are (w, x, y, z); squared norm summed in storage order x, y, z, w.
PW_HD void quat_normalize(const double *qin, double *q)
{
	const double w = qin[0], x = qin[1], y = qin[2], z = qin[3];
	const double n2 = add(add(add(mul(x, x), mul(y, y)), mul(z, z)), mul(w, w));
	if (n2 > 0.0) {
		const double n = rt(n2);
		q[0] = dvd(w, n); q[1] = dvd(x, n); q[2] = dvd(y, n); q[3] = dvd(z, n);
	} else {
		q[0] = w; q[1] = x; q[2] = y; q[3] = z;
	}
}

// Unit-quaternion rotation formula applied to raw coefficients (w, x, y, z).
PW_HD void quat_to_matrix(const double *q, double *R)
{
	const double w = q[0], x = q[1], y = q[2], z = q[3];
	const double tx = mul(2.0, x), ty = mul(2.0, y), tz = mul(2.0, z);
	const double twx = mul(tx, w), twy = mul(ty, w), twz = mul(tz, w);
	const double txx = mul(tx, x), txy = mul(ty, x), txz = mul(tz, x);
	const double tyy = mul(ty, y), tyz = mul(tz, y), tzz = mul(tz, z);
	R[0] = sub(1.0, add(tyy, tzz)); R[1] = sub(txy, twz);           R[2] = add(txz, twy);
	R[3] = add(txy, twz);           R[4] = sub(1.0, add(txx, tzz)); R[5] = sub(tyz, twx);
	R[6] = sub(txz, twy);           R[7] = add(tyz, twx);           R[8] = sub(1.0, add(txx, tyy));
}

PW_HD void xform_point(const double *R, const double *t, const double *p, double *o)
{
#pragma unroll
	for (int i = 0; i < 3; i++) {
		double s = mul(R[3 * i + 0], p[0]);
		s = add(s, mul(R[3 * i + 1], p[1]));
		s = add(s, mul(R[3 * i + 2], p[2]));
		o[i] = add(s, t[i]);
	}
}

PW_HD void state_transform(const double *q, double *R, double *t)
{
	const double quat[4] = { q[3], q[4], q[5], q[6] };
	quat_to_matrix(quat, R);
	t[0] = q[0]; t[1] = q[1]; t[2] = q[2];
}

// a * conj(b)
PW_HD void quat_mul_conj(const double *a, const double *b, double *o)
{
	const double bw = b[0], bx = -b[1], by = -b[2], bz = -b[3];
	o[0] = sub(sub(sub(mul(a[0], bw), mul(a[1], bx)), mul(a[2], by)), mul(a[3], bz));
	o[1] = sub(add(add(mul(a[0], bx), mul(a[1], bw)), mul(a[2], bz)), mul(a[3], by));
	o[2] = add(add(sub(mul(a[0], by), mul(a[1], bz)), mul(a[2], bw)), mul(a[3], bx));
	o[3] = add(sub(add(mul(a[0], bz), mul(a[1], by)), mul(a[2], bx)), mul(a[3], bw));
}

PW_HD double angular_distance(const double *a, const double *b)
{
	double d[4];
	quat_mul_conj(a, b, d);
	const double vn = rt(add(add(mul(d[1], d[1]), mul(d[2], d[2])), mul(d[3], d[3])));
	return mul(2.0, atan2q(vn, dabs(d[0])));
}

PW_HD double distance(const double *a, const double *b)
{
	double qa[4], qb[4];
	const double ra[4] = { a[3], a[4], a[5], a[6] };
	const double rb[4] = { b[3], b[4], b[5], b[6] };
	quat_normalize(ra, qa);
	quat_normalize(rb, qb);
	const double dx = sub(a[0], b[0]), dy = sub(a[1], b[1]), dz = sub(a[2], b[2]);
	const double tr = rt(add(add(mul(dx, dx), mul(dy, dy)), mul(dz, dz)));
	return add(tr, angular_distance(qa, qb));
}

// Per-segment constants of the interpolation: normalised rotations, their dot,
// the slerp angle and its sine (theta / sin only used when !linear).
struct SlerpParams {
	double qa[4], qb[4];
	double d, theta, stheta;
	int linear;
};

PW_HD void slerp_setup(const double *a, const double *b, SlerpParams &P)
{
	const double ra[4] = { a[3], a[4], a[5], a[6] };
	const double rb[4] = { b[3], b[4], b[5], b[6] };
	quat_normalize(ra, P.qa);
	quat_normalize(rb, P.qb);
	P.d = add(add(add(mul(P.qa[1], P.qb[1]), mul(P.qa[2], P.qb[2])), mul(P.qa[3], P.qb[3])), mul(P.qa[0], P.qb[0]));
	const double absd = dabs(P.d);
	P.linear = absd >= SLERP_ONE;
	if (!P.linear) {
		P.theta = acos01(absd);
		P.stheta = sin_q(P.theta);
	} else {
		P.theta = 0.0;
		P.stheta = 0.0;
	}
}

// interpolate(a, b, tau) given the segment's slerp constants.
PW_HD void interpolate_p(const double *a, const double *b, const SlerpParams &P, double tau, double *out)
{
	const double omt = sub(1.0, tau);
#pragma unroll
	for (int i = 0; i < 3; i++)
		out[i] = add(mul(a[i], omt), mul(b[i], tau));
	double s0, s1;
	if (P.linear) {
		s0 = omt;
		s1 = tau;
	} else {
		s0 = dvd(sin_q(mul(omt, P.theta)), P.stheta);
		s1 = dvd(sin_q(mul(tau, P.theta)), P.stheta);
	}
	if (P.d < 0.0)
		s1 = -s1;
#pragma unroll
	for (int i = 0; i < 4; i++)
		out[3 + i] = add(mul(s0, P.qa[i]), mul(s1, P.qb[i]));
}

// The same state for frames that only feed the certified FP32 filters: the
// slerp weights multiplied by inv_stheta = 1 / stheta instead of divided by
// stheta (two FP64 divisions fewer), the sines and the rotation's combination
// evaluated with fused multiply-adds (sin_qf).  On the slerp branch theta <=
// pi / 2, so each weight is at most 1 and lies within 2^-49 of the reference's;
// with unit rotations qa, qb the rotation's components lie within 2^-47 of the
// reference's and the raw-quaternion rotation matrix's entries within 2^-43.
// The filters' frames allow one more unit of 2^-24 for it (pwf::make_qf's
// state_ulps); tests/harness/delta_walk.cc checks the stated bounds against
// the reference's interpolation.  The translation is the reference's.
PW_HD void interpolate_w(const double *a, const double *b, const SlerpParams &P, double inv_stheta, double tau,
                         double *out)
{
	const double omt = sub(1.0, tau);
#pragma unroll
	for (int i = 0; i < 3; i++)
		out[i] = add(mul(a[i], omt), mul(b[i], tau));
	double s0, s1;
	if (P.linear) {
		s0 = omt;
		s1 = tau;
	} else {
		s0 = mul(sin_qf(mul(omt, P.theta)), inv_stheta);
		s1 = mul(sin_qf(mul(tau, P.theta)), inv_stheta);
	}
	if (P.d < 0.0)
		s1 = -s1;
#pragma unroll
	for (int i = 0; i < 4; i++)
		out[3 + i] = fmad(s1, P.qb[i], mul(s0, P.qa[i]));
}

PW_HD void interpolate(const double *a, const double *b, double tau, double *out)
{
	SlerpParams P;
	slerp_setup(a, b, P);
	interpolate_p(a, b, P, tau, out);
}

// One iteration of the reference's delta update (unit_world.cc:463-470).
PW_HD double advance_delta(double delta, double dist, double step)
{
	if (delta < dist) {
		delta = add(delta, step);
		return dist < delta ? dist : delta;
	}
	return add(delta, step);
}

PW_HD uint64_t dbits(double x)
{
	uint64_t b;
	memcpy(&b, &x, 8);
	return b;
}
PW_HD double bitsd(uint64_t b)
{
	double x;
	memcpy(&x, &b, 8);
	return x;
}

// How many of the next (at most jmax) iterations of advance_delta from `delta`
// can be taken at once, and their common increment *c: 0 when none.
//
// While delta stays in its binade [2^e, 2^(e+1)) it lies on the grid of
// u = ulp(delta), and every rounded sum fl(delta + step) equals delta + c with
// c = step rounded to a multiple of u (the grid is invariant under the shift by
// delta), unless step / u falls exactly halfway between two integers (a tie,
// whose rounding to even depends on delta: no jump then).  So k iterations give
// delta + k c exactly (k c and the sum are multiples of u below 2^(e+1)), as
// long as every exact sum stays inside the binade (delta + (k-1) c + step <=
// 2^(e+1)) and no result passes dist (delta + k c <= dist: the clamp of the
// reference loop is then never taken).  Both conditions are checked exactly.
// The tie test and u work on the bit patterns; c is fl(delta + step) - delta
// (exact); the run length is estimated in FP32 and only ever lowered, so the
// FP64 work is a handful of adds and multiplies (no division).
PW_HD int delta_jump(double delta, double dist, double step, int jmax, double *c)
{
	const uint64_t db = dbits(delta), sb = dbits(step);
	const int64_t ed = (int64_t)(db >> 52), es = (int64_t)(sb >> 52);   // biased exponents (both positive)
	if (!(delta > 0.0) || !(step > 0.0) || jmax <= 0 || ed < 60 || ed > 2000 || es == 0)
		return 0;
	// step = ms * 2^(es - 1075) with the 53-bit integer mantissa ms; u = 2^(ed - 1075)
	const int64_t k = ed - es;                 // step / u = ms / 2^k
	if (k > 53)
		return 0;                              // step below half an ulp of delta: it never moves delta
	if (k >= 1) {
		const uint64_t ms = (sb & 0x000FFFFFFFFFFFFFull) | 0x0010000000000000ull;
		if ((ms & ((uint64_t(1) << k) - 1u)) == (uint64_t(1) << (k - 1)))
			return 0;                          // a tie
	}
	const double top = bitsd((uint64_t)(ed + 1) << 52);   // 2^(e+1)
	const double cc = sub(add(delta, step), delta);
	if (!(cc > 0.0))
		return 0;
	// estimates of the two bounds (relative error below 4e-7: two roundings to FP32 and
	// one correctly rounded division), lowered by 1e-6 before the floor, so that the
	// count never exceeds the exact bound and the products below are exact
	const float fc = (float)cc;
	const float ka = (float)sub(sub(top, delta), step) / fc + 1.f;
	const float kb = (float)sub(dist, delta) / fc;
	float kf = fminf(fminf(ka, kb), (float)jmax);
	kf = kf * (1.f - 1e-6f);
	if (!(kf >= 1.f))
		return 0;
	int n = kf >= 2147483520.f ? 2147483520 : (int)kf;
	n = n < jmax ? n : jmax;
	const double last = add(delta, mul((double)(n - 1), cc));   // exact when the bounds hold
	if (!(step <= sub(top, last) && add(last, cc) <= dist))
		return 0;
	*c = cc;
	return n;
}

// Exactly k iterations of advance_delta from `delta` taken at once, when they stay
// inside delta's binade, meet no rounding tie and end at or below dist: then
// *res = delta + k c (c as for delta_jump) and the result is true.  No estimate
// is needed: last = delta + (k-1) c is exact whenever it stays below 2^(e+1); if
// (k-1) c or the sum rounds, the exact value is already at or above 2^(e+1), the
// rounded one too (rounding is monotone and 2^(e+1) is representable), and the
// binade test fails as it must.  For a constant k the FP64 work is two adds, a
// subtract, a multiply by a constant and two compares.
PW_HD bool delta_try(double delta, double dist, double step, int k, double *res)
{
	const uint64_t db = dbits(delta), sb = dbits(step);
	const int64_t ed = (int64_t)(db >> 52), es = (int64_t)(sb >> 52);
	if (!(delta > 0.0) || !(step > 0.0) || k <= 0 || ed < 60 || ed > 2000 || es == 0)
		return false;
	const int64_t sh = ed - es;
	if (sh > 53)
		return false;
	if (sh >= 1) {
		const uint64_t ms = (sb & 0x000FFFFFFFFFFFFFull) | 0x0010000000000000ull;
		if ((ms & ((uint64_t(1) << sh) - 1u)) == (uint64_t(1) << (sh - 1)))
			return false;                      // a tie
	}
	const double top = bitsd((uint64_t)(ed + 1) << 52);
	const double cc = sub(add(delta, step), delta);
	if (!(cc > 0.0))
		return false;
	const double last = add(delta, mul((double)(k - 1), cc));
	if (!(step <= sub(top, last)))
		return false;
	const double r = add(last, cc);
	if (!(r <= dist))
		return false;
	*res = r;
	return true;
}

// delta after j iterations of advance_delta, bit-identical to running them one
// by one: the whole run at once where delta_try allows it, otherwise one
// iteration and a new try (a run that crosses a binade boundary or meets dist).
PW_HD double walk_delta(double delta, double dist, double step, int j)
{
	while (j > 0) {
		double r;
		if (delta_try(delta, dist, step, j, &r))
			return r;
		delta = advance_delta(delta, dist, step);
		j--;
	}
	return delta;
}

// Eigenvectors (rows of E, orthonormal) of the symmetric 3 x 3 matrix S (xx, yy, zz,
// xy, xz, yz) by cyclic Jacobi rotations; the principal axes of an oriented node box.
// Plain FP64 (any orthonormal frame gives a valid box: accuracy only tightens it).
PW_HD void jacobi_eigen3(const double S[6], double E[9])
{
	double a[3][3] = { { S[0], S[3], S[4] }, { S[3], S[1], S[5] }, { S[4], S[5], S[2] } };
	double v[3][3] = { { 1, 0, 0 }, { 0, 1, 0 }, { 0, 0, 1 } };
	for (int sweep = 0; sweep < 32; sweep++) {
		const double off = fabs(a[0][1]) + fabs(a[0][2]) + fabs(a[1][2]);
		const double dia = fabs(a[0][0]) + fabs(a[1][1]) + fabs(a[2][2]);
		if (!(off > 1e-300) || off <= 1e-18 * dia)
			break;
		for (int p = 0; p < 2; p++)
			for (int q = p + 1; q < 3; q++) {
				if (!(fabs(a[p][q]) > 1e-300))
					continue;
				const double th = (a[q][q] - a[p][p]) / (2.0 * a[p][q]);
				const double t = (th >= 0.0 ? 1.0 : -1.0) / (fabs(th) + sqrt(th * th + 1.0));
				const double c = 1.0 / sqrt(t * t + 1.0), s = t * c;
				for (int k = 0; k < 3; k++) {
					const double akp = a[k][p], akq = a[k][q];
					a[k][p] = c * akp - s * akq;
					a[k][q] = s * akp + c * akq;
				}
				for (int k = 0; k < 3; k++) {
					const double apk = a[p][k], aqk = a[q][k];
					a[p][k] = c * apk - s * aqk;
					a[q][k] = s * apk + c * aqk;
				}
				for (int k = 0; k < 3; k++) {
					const double vkp = v[k][p], vkq = v[k][q];
					v[k][p] = c * vkp - s * vkq;
					v[k][q] = s * vkp + c * vkq;
				}
			}
	}
	// columns of v are the eigenvectors; re-orthonormalise (Gram-Schmidt, then a cross product)
	double e0[3] = { v[0][0], v[1][0], v[2][0] }, e1[3] = { v[0][1], v[1][1], v[2][1] };
	const double n0 = sqrt(e0[0] * e0[0] + e0[1] * e0[1] + e0[2] * e0[2]);
	for (int k = 0; k < 3; k++) e0[k] /= n0;
	const double d = e0[0] * e1[0] + e0[1] * e1[1] + e0[2] * e1[2];
	for (int k = 0; k < 3; k++) e1[k] -= d * e0[k];
	const double n1 = sqrt(e1[0] * e1[0] + e1[1] * e1[1] + e1[2] * e1[2]);
	if (!(n1 > 1e-6)) {
		// a degenerate pair (never for Jacobi's orthogonal output): any perpendicular unit vector
		const int m = fabs(e0[0]) < 0.6 ? 0 : 1;
		double u[3] = { 0, 0, 0 };
		u[m] = 1.0;
		const double du = e0[m];
		for (int k = 0; k < 3; k++) e1[k] = u[k] - du * e0[k];
		const double nn = sqrt(e1[0] * e1[0] + e1[1] * e1[1] + e1[2] * e1[2]);
		for (int k = 0; k < 3; k++) e1[k] /= nn;
	} else {
		for (int k = 0; k < 3; k++) e1[k] /= n1;
	}
	E[0] = e0[0]; E[1] = e0[1]; E[2] = e0[2];
	E[3] = e1[0]; E[4] = e1[1]; E[5] = e1[2];
	E[6] = e0[1] * e1[2] - e0[2] * e1[1];
	E[7] = e0[2] * e1[0] - e0[0] * e1[2];
	E[8] = e0[0] * e1[1] - e0[1] * e1[0];
}

// ---------------------------------------------------------------- Moeller

PW_HD void sub3(const double *a, const double *b, double *o)
{
	o[0] = sub(a[0], b[0]); o[1] = sub(a[1], b[1]); o[2] = sub(a[2], b[2]);
}
PW_HD void cross3(const double *a, const double *b, double *o)
{
	o[0] = sub(mul(a[1], b[2]), mul(a[2], b[1]));
	o[1] = sub(mul(a[2], b[0]), mul(a[0], b[2]));
	o[2] = sub(mul(a[0], b[1]), mul(a[1], b[0]));
}
PW_HD double dot3(const double *a, const double *b)
{
	return add(add(mul(a[0], b[0]), mul(a[1], b[1])), mul(a[2], b[2]));
}

PW_HD int edge_edge(double ax, double ay, const double *v0, const double *u0, const double *u1, int i0, int i1)
{
	const double bx = sub(u0[i0], u1[i0]);
	const double by = sub(u0[i1], u1[i1]);
	const double cx = sub(v0[i0], u0[i0]);
	const double cy = sub(v0[i1], u0[i1]);
	const double f = sub(mul(ay, bx), mul(ax, by));
	const double d = sub(mul(by, cx), mul(bx, cy));
	if ((f > 0.0 && d >= 0.0 && d <= f) || (f < 0.0 && d <= 0.0 && d >= f)) {
		const double e = sub(mul(ax, cy), mul(ay, cx));
		if (f > 0.0) {
			if (e >= 0.0 && e <= f)
				return 1;
		} else {
			if (e <= 0.0 && e >= f)
				return 1;
		}
	}
	return 0;
}

PW_HD int edge_against_tri(const double *v0, const double *v1, const double *const *U, int i0, int i1)
{
	const double ax = sub(v1[i0], v0[i0]);
	const double ay = sub(v1[i1], v0[i1]);
	if (edge_edge(ax, ay, v0, U[0], U[1], i0, i1)) return 1;
	if (edge_edge(ax, ay, v0, U[1], U[2], i0, i1)) return 1;
	if (edge_edge(ax, ay, v0, U[2], U[0], i0, i1)) return 1;
	return 0;
}

PW_HD int point_in_tri(const double *p, const double *const *U, int i0, int i1)
{
	double dd[3];
#pragma unroll
	for (int k = 0; k < 3; k++) {
		const double *a0 = U[k];
		const double *a1 = U[k == 2 ? 0 : k + 1];
		const double a = sub(a1[i1], a0[i1]);
		const double b = -sub(a1[i0], a0[i0]);
		const double c = sub(mul(-a, a0[i0]), mul(b, a0[i1]));
		dd[k] = add(add(mul(a, p[i0]), mul(b, p[i1])), c);
	}
	return (mul(dd[0], dd[1]) > 0.0 && mul(dd[0], dd[2]) > 0.0) ? 1 : 0;
}

PW_HD int coplanar_test(const double *N, const double *const *V, const double *const *U)
{
	const double a0 = dabs(N[0]), a1 = dabs(N[1]), a2 = dabs(N[2]);
	int i0, i1;
	if (a0 > a1) {
		if (a0 > a2) { i0 = 1; i1 = 2; }
		else         { i0 = 0; i1 = 1; }
	} else {
		if (a2 > a1) { i0 = 0; i1 = 1; }
		else         { i0 = 0; i1 = 2; }
	}
	if (edge_against_tri(V[0], V[1], U, i0, i1)) return 1;
	if (edge_against_tri(V[1], V[2], U, i0, i1)) return 1;
	if (edge_against_tri(V[2], V[0], U, i0, i1)) return 1;
	if (point_in_tri(V[0], U, i0, i1)) return 1;
	if (point_in_tri(U[0], V, i0, i1)) return 1;
	return 0;
}

PW_HD void plane_dists(const double *const *S, const double *const *T, double eps, double *N, double *dist)
{
	double e1[3], e2[3];
	sub3(S[1], S[0], e1);
	sub3(S[2], S[0], e2);
	cross3(e1, e2, N);
	const double d = -dot3(N, S[0]);
#pragma unroll
	for (int k = 0; k < 3; k++) {
		double v = add(dot3(N, T[k]), d);
		if (dabs(v) < eps)
			v = 0.0;
		dist[k] = v;
	}
}

PW_HD int lone_vertex(const double *D)
{
	if (mul(D[0], D[1]) > 0.0) return 2;
	if (mul(D[0], D[2]) > 0.0) return 1;
	if (mul(D[1], D[2]) > 0.0 || D[0] != 0.0) return 0;
	if (D[1] != 0.0) return 1;
	if (D[2] != 0.0) return 2;
	return -1;
}

PW_HD void others(int lone, int &o1, int &o2)
{
	if (lone == 0) { o1 = 1; o2 = 2; }
	else if (lone == 1) { o1 = 0; o2 = 2; }
	else { o1 = 0; o2 = 1; }
}

PW_HD int max_axis(const double *D)
{
	double m = dabs(D[0]);
	int idx = 0;
	const double b = dabs(D[1]), c = dabs(D[2]);
	if (b > m) { m = b; idx = 1; }
	if (c > m) { m = c; idx = 2; }
	return idx;
}

PW_HD void interval(const double *const *T, const double *D, int lone, int ax, double *out)
{
	int o1, o2;
	others(lone, o1, o2);
	const double pl = T[lone][ax];
	out[0] = add(pl, dvd(mul(sub(T[o1][ax], pl), D[lone]), sub(D[lone], D[o1])));
	out[1] = add(pl, dvd(mul(sub(T[o2][ax], pl), D[lone]), sub(D[lone], D[o2])));
}

// Boolean test: V = env triangle (first), U = robot triangle (second).
PW_HD int tri_tri(const double *V0, const double *V1, const double *V2,
                  const double *U0, const double *U1, const double *U2, double eps)
{
	const double *V[3] = { V0, V1, V2 };
	const double *U[3] = { U0, U1, U2 };
	double N1[3], N2[3], du[3], dv[3];
	plane_dists(V, U, eps, N1, du);
	if (mul(du[0], du[1]) > 0.0 && mul(du[0], du[2]) > 0.0)
		return 0;
	plane_dists(U, V, eps, N2, dv);
	if (mul(dv[0], dv[1]) > 0.0 && mul(dv[0], dv[2]) > 0.0)
		return 0;
	double Dl[3];
	cross3(N1, N2, Dl);
	const int ax = max_axis(Dl);
	const int lv = lone_vertex(dv);
	if (lv < 0)
		return coplanar_test(N1, V, U);
	const int lu = lone_vertex(du);
	if (lu < 0)
		return coplanar_test(N1, V, U);
	double iv[2], iu[2];
	interval(V, dv, lv, ax, iv);
	interval(U, du, lu, ax, iu);
	if (iv[0] > iv[1]) { const double c = iv[0]; iv[0] = iv[1]; iv[1] = c; }
	if (iu[0] > iu[1]) { const double c = iu[0]; iu[0] = iu[1]; iu[1] = c; }
	if (iv[1] < iu[0] || iu[1] < iv[0])
		return 0;
	return 1;
}

PW_HD void interval_pts(const double *const *T, const double *D, int lone, int ax,
                        double *iv, double *p0, double *p1)
{
	int o1, o2;
	others(lone, o1, o2);
	const double *A = T[lone];
	const double pl = A[ax];
	double r = dvd(D[lone], sub(D[lone], D[o1]));
	iv[0] = add(pl, mul(sub(T[o1][ax], pl), r));
#pragma unroll
	for (int c = 0; c < 3; c++)
		p0[c] = add(mul(sub(T[o1][c], A[c]), r), A[c]);
	r = dvd(D[lone], sub(D[lone], D[o2]));
	iv[1] = add(pl, mul(sub(T[o2][ax], pl), r));
#pragma unroll
	for (int c = 0; c < 3; c++)
		p1[c] = add(A[c], mul(sub(T[o2][c], A[c]), r));
}

// Test with the intersection segment (Moeller's 2001 extension).  Points are
// zero for misses and coplanar pairs.
PW_HD int tri_tri_isect(const double *V0, const double *V1, const double *V2,
                        const double *U0, const double *U1, const double *U2, double eps,
                        int *coplanar, double *pt1, double *pt2)
{
	const double *V[3] = { V0, V1, V2 };
	const double *U[3] = { U0, U1, U2 };
	double N1[3], N2[3], du[3], dv[3];
	*coplanar = 0;
	for (int c = 0; c < 3; c++) { pt1[c] = 0.0; pt2[c] = 0.0; }
	plane_dists(V, U, eps, N1, du);
	if (mul(du[0], du[1]) > 0.0 && mul(du[0], du[2]) > 0.0)
		return 0;
	plane_dists(U, V, eps, N2, dv);
	if (mul(dv[0], dv[1]) > 0.0 && mul(dv[0], dv[2]) > 0.0)
		return 0;
	double Dl[3];
	cross3(N1, N2, Dl);
	const int ax = max_axis(Dl);
	const int lv = lone_vertex(dv);
	if (lv < 0) {
		*coplanar = 1;
		return coplanar_test(N1, V, U);
	}
	const int lu = lone_vertex(du);
	if (lu < 0) {
		*coplanar = 1;
		return coplanar_test(N1, V, U);
	}
	double iv[2], iu[2], a1[3], a2[3], b1[3], b2[3];
	interval_pts(V, dv, lv, ax, iv, a1, a2);
	interval_pts(U, du, lu, ax, iu, b1, b2);
	int sv = 0, su = 0;
	if (iv[0] > iv[1]) { const double c = iv[0]; iv[0] = iv[1]; iv[1] = c; sv = 1; }
	if (iu[0] > iu[1]) { const double c = iu[0]; iu[0] = iu[1]; iu[1] = c; su = 1; }
	if (iv[1] < iu[0] || iu[1] < iv[0])
		return 0;
	const double *s, *e;
	if (iu[0] < iv[0]) {
		s = sv ? a2 : a1;
		if (iu[1] < iv[1]) e = su ? b1 : b2;
		else               e = sv ? a1 : a2;
	} else {
		s = su ? b2 : b1;
		if (iu[1] > iv[1]) e = sv ? a1 : a2;
		else               e = su ? b1 : b2;
	}
	for (int c = 0; c < 3; c++) { pt1[c] = s[c]; pt2[c] = e[c]; }
	return 1;
}

// ---------------------------------------------------------------- boxes

// Separating-axis test of an axis-aligned box (half-extents ea) against a box
// with axes = columns of R, half-extents eb, centre offset T; AR = |R| + slack.
// 1 = a separating axis exists (strict), 0 = overlap or touch.
PW_HD int sat_disjoint(const double *ea, const double *eb, const double *T, const double *R, const double *AR)
{
	for (int i = 0; i < 3; i++) {
		const double rb = add(add(mul(eb[0], AR[3 * i + 0]), mul(eb[1], AR[3 * i + 1])), mul(eb[2], AR[3 * i + 2]));
		if (dabs(T[i]) > add(ea[i], rb)) return 1;
	}
	for (int j = 0; j < 3; j++) {
		const double tl = add(add(mul(T[0], R[0 + j]), mul(T[1], R[3 + j])), mul(T[2], R[6 + j]));
		const double ra = add(add(mul(ea[0], AR[0 + j]), mul(ea[1], AR[3 + j])), mul(ea[2], AR[6 + j]));
		if (dabs(tl) > add(ra, eb[j])) return 1;
	}
	for (int i = 0; i < 3; i++) {
		const int i1 = (i + 1) % 3, i2 = (i + 2) % 3;
		for (int j = 0; j < 3; j++) {
			const int j1 = (j + 1) % 3, j2 = (j + 2) % 3;
			const double tl = sub(mul(T[i2], R[3 * i1 + j]), mul(T[i1], R[3 * i2 + j]));
			const double ra = add(mul(ea[i1], AR[3 * i2 + j]), mul(ea[i2], AR[3 * i1 + j]));
			const double rb = add(mul(eb[j1], AR[3 * i + j2]), mul(eb[j2], AR[3 * i + j1]));
			if (dabs(tl) > add(ra, rb)) return 1;
		}
	}
	return 0;
}

// isDisentangled box test with the env box's centre already placed, ce = Re ec + te.
// ROT = false takes Re as exactly the identity: for a finite state Re^T d and
// Re^T R then equal d and R up to the sign of zeros (products by 1, sums with
// products by 0), which no comparison of the test sees; callers use it only
// for finite states (a non-finite one gives NaN products in the general form).
template <bool ROT = true>
PW_HD int boxes_disjoint_placed(const double *q, const double *rc, const double *rh, const double *Re,
                                const double *ce, const double *eh)
{
	double R[9], t[3], cr[3], d[3], Rr[9], T[3], AR[9];
	state_transform(q, R, t);
	xform_point(R, t, rc, cr);
	for (int c = 0; c < 3; c++) d[c] = sub(cr[c], ce[c]);
	for (int i = 0; i < 3; i++) {
		T[i] = ROT ? add(add(mul(Re[0 + i], d[0]), mul(Re[3 + i], d[1])), mul(Re[6 + i], d[2])) : d[i];
		for (int j = 0; j < 3; j++)
			Rr[3 * i + j] = ROT ? add(add(mul(Re[0 + i], R[0 + j]), mul(Re[3 + i], R[3 + j])), mul(Re[6 + i], R[6 + j]))
			                    : R[3 * i + j];
	}
	for (int i = 0; i < 9; i++) AR[i] = dabs(Rr[i]);
	return sat_disjoint(eh, rh, T, Rr, AR);
}

// isDisentangled box test: robot local AABB box (rc, rh) placed by the state,
// env box (ec, eh) placed by the perturbation transform (Re, te).
PW_HD int boxes_disjoint(const double *q, const double *rc, const double *rh,
                         const double *Re, const double *te, const double *ec, const double *eh)
{
	double ce[3];
	xform_point(Re, te, ec, ce);
	return boxes_disjoint_placed(q, rc, rh, Re, ce, eh);
}

// ---------------------------------------------------------------- key configurations
//
// UnitWorld::enumFreeConfiguration / sampleFreeConfiguration
// (lib/osr/unit_world.cc:1294-1389) place the robot so that its surface point
// plus margin x normal meets the environment's, normals opposed, then spin it
// about the environment normal.  Eigen's published forms, each operation
// rounded on its own, in the order written:
//   shortest arc a -> b (Quaternion::setFromTwoVectors): v0 = a / |a|,
//     v1 = b / |b|, c = v0 . v1; w = s / 2, vec = (v0 x v1) * (1 / s) with
//     s = sqrt((1 + c) * 2); for c < -1 + 1e-12 a half turn about a unit axis
//     perpendicular to v0 (v0 x the basis vector of its smallest |component|);
//   angle-axis (AngleAxis -> Quaternion): (cos(angle / 2), sin(angle / 2) * axis),
//     the half-angle cosine and sine given (computed once on the host);
//   rotation of v (Quaternion * vector): t = u x v, t = t + t, v + w t + u x t;
//   compose: translation, quaternion normalised (quat_normalize).

// |v| with the sum of squares in index order.
PW_HD double norm3(const double *v) { return rt(add(add(mul(v[0], v[0]), mul(v[1], v[1])), mul(v[2], v[2]))); }

// Shortest-arc rotation (w, x, y, z) taking direction a to direction b.
PW_HD void shortest_arc(const double *a, const double *b, double *q)
{
	const double na = norm3(a), nb = norm3(b);
	const double v0[3] = { dvd(a[0], na), dvd(a[1], na), dvd(a[2], na) };
	const double v1[3] = { dvd(b[0], nb), dvd(b[1], nb), dvd(b[2], nb) };
	const double c = add(add(mul(v0[0], v1[0]), mul(v0[1], v1[1])), mul(v0[2], v1[2]));
	if (c < -1.0 + 1e-12) {
		int k = 0;
		if (dabs(v0[1]) < dabs(v0[k]))
			k = 1;
		if (dabs(v0[2]) < dabs(v0[k]))
			k = 2;
		const double e[3] = { k == 0 ? 1.0 : 0.0, k == 1 ? 1.0 : 0.0, k == 2 ? 1.0 : 0.0 };
		double ax[3];
		cross3(v0, e, ax);
		const double n = norm3(ax);
		q[0] = 0.0;
		q[1] = dvd(ax[0], n);
		q[2] = dvd(ax[1], n);
		q[3] = dvd(ax[2], n);
		return;
	}
	const double s = rt(mul(add(1.0, c), 2.0));
	const double invs = dvd(1.0, s);
	double ax[3];
	cross3(v0, v1, ax);
	q[0] = mul(s, 0.5);
	q[1] = mul(ax[0], invs);
	q[2] = mul(ax[1], invs);
	q[3] = mul(ax[2], invs);
}

// Hamilton product a * b of (w, x, y, z) quaternions, each sum left to right.
PW_HD void quat_mul(const double *a, const double *b, double *o)
{
	o[0] = sub(sub(sub(mul(a[0], b[0]), mul(a[1], b[1])), mul(a[2], b[2])), mul(a[3], b[3]));
	o[1] = sub(add(add(mul(a[0], b[1]), mul(a[1], b[0])), mul(a[2], b[3])), mul(a[3], b[2]));
	o[2] = add(add(sub(mul(a[0], b[2]), mul(a[1], b[3])), mul(a[2], b[0])), mul(a[3], b[1]));
	o[3] = add(sub(add(mul(a[0], b[3]), mul(a[1], b[2])), mul(a[2], b[1])), mul(a[3], b[0]));
}

// v rotated by the quaternion q (w, x, y, z), unnormalised formula.
PW_HD void quat_rotate(const double *q, const double *v, double *o)
{
	const double u[3] = { q[1], q[2], q[3] };
	double t[3], ut[3];
	cross3(u, v, t);
	t[0] = add(t[0], t[0]);
	t[1] = add(t[1], t[1]);
	t[2] = add(t[2], t[2]);
	cross3(u, t, ut);
	for (int i = 0; i < 3; i++)
		o[i] = add(add(v[i], mul(q[0], t[i])), ut[i]);
}

// The key-configuration state of one surface pair and one spin (half-angle
// cosine hc and sine hs of the spin about the environment normal).
PW_HD void keyconf_state(const double *rp, const double *rn, const double *ep, const double *en, double margin,
                         double hc, double hs, double *out)
{
	double rob_o[3], env_o[3], neg_en[3];
	for (int i = 0; i < 3; i++) {
		rob_o[i] = add(rp[i], mul(rn[i], margin));
		env_o[i] = add(ep[i], mul(en[i], margin));
		neg_en[i] = -en[i];
	}
	double r1[4], acc[4], rv[3];
	shortest_arc(rn, neg_en, r1);
	const double r2[4] = { hc, mul(hs, en[0]), mul(hs, en[1]), mul(hs, en[2]) };
	quat_mul(r2, r1, acc);
	quat_rotate(acc, rob_o, rv);
	for (int i = 0; i < 3; i++)
		out[i] = sub(env_o[i], rv[i]);
	quat_normalize(acc, out + 3);
}

} // namespace pwm
