/*
 * pw_oracle.c -- CPU oracle for the collision-query path of pyosr's UnitWorld.
 *
 * TEST INFRASTRUCTURE ONLY.  Nothing in the product library links, loads or
 * calls this file.  Only tests/, __graft_entry__.smoke() and the CPU-baseline
 * leg of bench.py use it, and only as the checker (or as the timed CPU
 * restatement of the reference path).
 *
 * It restates, in plain C99 with IEEE double arithmetic and no FMA contraction
 * (build with -ffp-contract=off), the reference's algorithm for:
 *   - the unit-world normalisation recipe
 *       lib/osr/unit_world.cc:123-161 (scaleToUnit, angleModel),
 *       lib/osr/scene.cc:78-156,211-229 (load, moveToCenter, scale),
 *       lib/osr/bbox.h:21-51 (bounding box seeded at the origin),
 *       lib/osr/cdmodel.cc:120-160 (addVF: float xform applied in double);
 *   - SE(3) state math, lib/osr/osr_state.cc:16-44 (transform, interpolate),
 *     :85-154 (decompose, compose, distance);
 *   - isValid / isDisentangled, lib/osr/unit_world.cc:197-264, with the
 *     box-box test of lib/osr/cdmodel.cc:85-114,180-197;
 *   - transitStateToWithContact / isValidTransition,
 *     lib/osr/unit_world.cc:405-486 (delta accumulation, clamps, early exit);
 *   - intersectingSegments, lib/osr/unit_world.cc:959-1012 with
 *     lib/tritri/tritri_igl.hh and Moeller's tri-tri test with intersection
 *     line (lib/tritri/Moller97d.cc:579).
 *
 * The reference's verdict arithmetic lives in FCL (fcl::collide on
 * BVHModel<OBBRSS<double>>, lib/osr/cdmodel.cc:171), which is an un-vendored
 * submodule of unknown commit.  Its triangle predicate cannot be restated
 * here.  This oracle uses Moeller's 1997 triangle-triangle test in FP64
 * without the coplanarity snap (epsilon 0) as the collision predicate, and
 * the reference's 1e-6 snap only for intersecting_segments, exactly as the
 * reference does there.  Parity with FCL's own predicate is therefore
 * UNPINNED for exactly-touching and coplanar configurations; everywhere else
 * the verdict is a property of the geometry, not of the BVH.
 *
 * Eigen's slerp / angularDistance and libm's sin/acos/atan2 are restated with
 * this file's own FP64 routines (Taylor series after half-angle and
 * complement argument reduction), so that results are reproducible bit for
 * bit on any IEEE machine.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define OR_EXPORT __attribute__((visibility("default")))

/* ------------------------------------------------------------------------ */
/* Deterministic FP64 elementary functions                                   */
/* ------------------------------------------------------------------------ */

static const double OR_PIO2_HI = 1.5707963267948965579989817342720925807952880859375;
static const double OR_PIO2_LO = 6.123233995736766035868820147291818e-17;
static const double OR_PIO4_HI = 0.78539816339744827899949086713604629039764404296875;
static const double OR_PIO4_LO = 3.061616997868383017934410073645909e-17;
static const double OR_TAN_PI_8 = 0.41421356237309503;

/* sin(x) for |x| <= pi/4: odd Taylor polynomial through x^17. */
static double or_sin_kernel(double x)
{
	const double z = x * x;
	double p = 2.8114572543455207632e-15;      /*  1/17! */
	p = p * z - 7.6471637318198164759e-13;      /* -1/15! */
	p = p * z + 1.6059043836821614599e-10;      /*  1/13! */
	p = p * z - 2.5052108385441718775e-08;      /* -1/11! */
	p = p * z + 2.7557319223985890653e-06;      /*  1/9!  */
	p = p * z - 1.9841269841269841270e-04;      /* -1/7!  */
	p = p * z + 8.3333333333333333333e-03;      /*  1/5!  */
	p = p * z - 1.6666666666666666667e-01;      /* -1/3!  */
	return x + x * (z * p);
}

/* cos(y) for |y| <= pi/4: even Taylor polynomial through y^18. */
static double or_cos_kernel(double y)
{
	const double z = y * y;
	double p = -1.5619206968586225271e-16;      /* -1/18! */
	p = p * z + 4.7794773323873852974e-14;      /*  1/16! */
	p = p * z - 1.1470745597729724714e-11;      /* -1/14! */
	p = p * z + 2.0876756987868098979e-09;      /*  1/12! */
	p = p * z - 2.7557319223985890653e-07;      /* -1/10! */
	p = p * z + 2.4801587301587301587e-05;      /*  1/8!  */
	p = p * z - 1.3888888888888888889e-03;      /* -1/6!  */
	p = p * z + 4.1666666666666666667e-02;      /*  1/4!  */
	p = p * z - 5.0000000000000000000e-01;      /* -1/2!  */
	return 1.0 + z * p;
}

/* sin(x) for x in [-pi/4, pi/2 + small]: the slerp angles never leave it. */
OR_EXPORT double or_sin(double x)
{
	if (x <= OR_PIO4_HI)
		return or_sin_kernel(x);
	const double y = (OR_PIO2_HI - x) + OR_PIO2_LO;
	return or_cos_kernel(y);
}

/* atan(z) for z in [0, 1]. */
static double or_atan01(double z)
{
	int shifted = 0;
	if (z > OR_TAN_PI_8) {
		/* atan(z) = pi/4 + atan((z - 1) / (z + 1)) */
		z = (z - 1.0) / (z + 1.0);
		shifted = 1;
	}
	/* half-angle: atan(z) = 2 atan(z / (1 + sqrt(1 + z^2))) */
	const double w = z / (1.0 + sqrt(1.0 + z * z));
	const double s = w * w;
	double p = 0.043478260869565216;
	p = p * s - 0.047619047619047616;
	p = p * s + 0.05263157894736842;
	p = p * s - 0.058823529411764705;
	p = p * s + 0.06666666666666667;
	p = p * s - 0.07692307692307693;
	p = p * s + 0.09090909090909091;
	p = p * s - 0.1111111111111111;
	p = p * s + 0.14285714285714285;
	p = p * s - 0.2;
	p = p * s + 0.3333333333333333;
	const double a = w - w * (s * p);
	double r = 2.0 * a;
	if (shifted)
		r = OR_PIO4_HI + (r + OR_PIO4_LO);
	return r;
}

/* atan2(y, x) for y >= 0, x >= 0 (first quadrant only). */
OR_EXPORT double or_atan2q(double y, double x)
{
	if (y == 0.0)
		return 0.0;
	if (y <= x)
		return or_atan01(y / x);
	return (OR_PIO2_HI - or_atan01(x / y)) + OR_PIO2_LO;
}

/* acos(a) for a in [0, 1]: acos(a) = 2 atan(sqrt(1 - a) / sqrt(1 + a)). */
OR_EXPORT double or_acos01(double a)
{
	const double y = sqrt(1.0 - a);
	const double x = sqrt(1.0 + a);
	return 2.0 * or_atan2q(y, x);
}

/* ------------------------------------------------------------------------ */
/* SE(3) state math.  State = [x, y, z, w, qx, qy, qz] (osr_state.h:20-33).  */
/* ------------------------------------------------------------------------ */

/* Normalise a quaternion given as (w, x, y, z); the squared norm is summed in
 * Eigen's storage order (x, y, z, w). */
static void or_quat_normalize(const double qin[4], double qout[4])
{
	const double w = qin[0], x = qin[1], y = qin[2], z = qin[3];
	const double n2 = ((x * x + y * y) + z * z) + w * w;
	if (n2 > 0.0) {
		const double n = sqrt(n2);
		qout[0] = w / n; qout[1] = x / n; qout[2] = y / n; qout[3] = z / n;
	} else {
		qout[0] = w; qout[1] = x; qout[2] = y; qout[3] = z;
	}
}

/* Rotation matrix of a (possibly un-normalised) quaternion (w, x, y, z),
 * the textbook unit-quaternion formula applied to the raw coefficients, as
 * translate_state_to_transform does (osr_state.cc:16-25). */
static void or_quat_to_matrix(const double q[4], double R[9])
{
	const double w = q[0], x = q[1], y = q[2], z = q[3];
	const double tx = 2.0 * x, ty = 2.0 * y, tz = 2.0 * z;
	const double twx = tx * w, twy = ty * w, twz = tz * w;
	const double txx = tx * x, txy = ty * x, txz = tz * x;
	const double tyy = ty * y, tyz = tz * y, tzz = tz * z;
	R[0] = 1.0 - (tyy + tzz); R[1] = txy - twz;         R[2] = txz + twy;
	R[3] = txy + twz;         R[4] = 1.0 - (txx + tzz); R[5] = tyz - twx;
	R[6] = txz - twy;         R[7] = tyz + twx;         R[8] = 1.0 - (txx + tyy);
}

/* p' = R p + t with the row sums taken left to right. */
static void or_xform_point(const double R[9], const double t[3], const double p[3], double out[3])
{
	for (int i = 0; i < 3; i++) {
		double s = R[3 * i + 0] * p[0];
		s = s + R[3 * i + 1] * p[1];
		s = s + R[3 * i + 2] * p[2];
		out[i] = s + t[i];
	}
}

static void or_state_transform(const double q[7], double R[9], double t[3])
{
	const double quat[4] = { q[3], q[4], q[5], q[6] };
	or_quat_to_matrix(quat, R);
	t[0] = q[0]; t[1] = q[1]; t[2] = q[2];
}

/* Hamilton product a * conj(b), both (w, x, y, z). */
static void or_quat_mul_conj(const double a[4], const double b[4], double o[4])
{
	const double bw = b[0], bx = -b[1], by = -b[2], bz = -b[3];
	o[0] = ((a[0] * bw - a[1] * bx) - a[2] * by) - a[3] * bz;
	o[1] = ((a[0] * bx + a[1] * bw) + a[2] * bz) - a[3] * by;
	o[2] = ((a[0] * by - a[1] * bz) + a[2] * bw) + a[3] * bx;
	o[3] = ((a[0] * bz + a[1] * by) - a[2] * bx) + a[3] * bw;
}

/* Rotation angle between two unit quaternions: 2 atan2(|v|, |w|) of a*conj(b). */
static double or_angular_distance(const double a[4], const double b[4])
{
	double d[4];
	or_quat_mul_conj(a, b, d);
	const double vn = sqrt((d[1] * d[1] + d[2] * d[2]) + d[3] * d[3]);
	return 2.0 * or_atan2q(vn, fabs(d[0]));
}

/* distance(), osr_state.cc:130-154: |dt| + angularDistance of the normalised rotations. */
OR_EXPORT double or_distance(const double a[7], const double b[7])
{
	double qa[4], qb[4];
	const double ra[4] = { a[3], a[4], a[5], a[6] };
	const double rb[4] = { b[3], b[4], b[5], b[6] };
	or_quat_normalize(ra, qa);
	or_quat_normalize(rb, qb);
	const double dx = a[0] - b[0], dy = a[1] - b[1], dz = a[2] - b[2];
	const double tr = sqrt((dx * dx + dy * dy) + dz * dz);
	return tr + or_angular_distance(qa, qb);
}

/* Slerp coefficients between two unit quaternions (Shoemake 1985), with the
 * linear fallback when |dot| >= 1 - 2^-52; s1 carries the sign of dot. */
static void or_slerp_coeffs(double d, double tau, double *s0, double *s1)
{
	const double absd = fabs(d);
	const double one = 1.0 - 2.220446049250313080847e-16;
	if (absd >= one) {
		*s0 = 1.0 - tau;
		*s1 = tau;
	} else {
		const double theta = or_acos01(absd);
		const double st = or_sin(theta);
		*s0 = or_sin((1.0 - tau) * theta) / st;
		*s1 = or_sin(tau * theta) / st;
	}
	if (d < 0.0)
		*s1 = -*s1;
}

/* interpolate(), osr_state.cc:27-44. */
OR_EXPORT void or_interpolate(const double a[7], const double b[7], double tau, double out[7])
{
	const double omt = 1.0 - tau;
	for (int i = 0; i < 3; i++)
		out[i] = a[i] * omt + b[i] * tau;
	double qa[4], qb[4];
	const double ra[4] = { a[3], a[4], a[5], a[6] };
	const double rb[4] = { b[3], b[4], b[5], b[6] };
	or_quat_normalize(ra, qa);
	or_quat_normalize(rb, qb);
	/* dot in storage order x, y, z, w */
	const double d = ((qa[1] * qb[1] + qa[2] * qb[2]) + qa[3] * qb[3]) + qa[0] * qb[0];
	double s0, s1;
	or_slerp_coeffs(d, tau, &s0, &s1);
	for (int i = 0; i < 4; i++)
		out[3 + i] = s0 * qa[i] + s1 * qb[i];
}

/* ------------------------------------------------------------------------ */
/* Moeller 1997 triangle-triangle test (restated from the JGT paper)         */
/* ------------------------------------------------------------------------ */

static void or_sub3(const double a[3], const double b[3], double o[3])
{
	o[0] = a[0] - b[0]; o[1] = a[1] - b[1]; o[2] = a[2] - b[2];
}
static void or_cross3(const double a[3], const double b[3], double o[3])
{
	o[0] = a[1] * b[2] - a[2] * b[1];
	o[1] = a[2] * b[0] - a[0] * b[2];
	o[2] = a[0] * b[1] - a[1] * b[0];
}
static double or_dot3(const double a[3], const double b[3])
{
	return (a[0] * b[0] + a[1] * b[1]) + a[2] * b[2];
}

/* Antonio's 2-D segment test (Graphics Gems III) of edge (v0 + A) against edge (u0, u1). */
static int or_edge_edge(double ax, double ay, const double v0[3], const double u0[3],
                        const double u1[3], int i0, int i1)
{
	const double bx = u0[i0] - u1[i0];
	const double by = u0[i1] - u1[i1];
	const double cx = v0[i0] - u0[i0];
	const double cy = v0[i1] - u0[i1];
	const double f = ay * bx - ax * by;
	const double d = by * cx - bx * cy;
	if ((f > 0.0 && d >= 0.0 && d <= f) || (f < 0.0 && d <= 0.0 && d >= f)) {
		const double e = ax * cy - ay * cx;
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

static int or_edge_against_tri(const double v0[3], const double v1[3], const double *U[3], int i0, int i1)
{
	const double ax = v1[i0] - v0[i0];
	const double ay = v1[i1] - v0[i1];
	if (or_edge_edge(ax, ay, v0, U[0], U[1], i0, i1)) return 1;
	if (or_edge_edge(ax, ay, v0, U[1], U[2], i0, i1)) return 1;
	if (or_edge_edge(ax, ay, v0, U[2], U[0], i0, i1)) return 1;
	return 0;
}

/* Is point p strictly on the same side of all three edges of triangle U (2-D)? */
static int or_point_in_tri(const double p[3], const double *U[3], int i0, int i1)
{
	double dd[3];
	for (int k = 0; k < 3; k++) {
		const double *a0 = U[k], *a1 = U[(k + 1) % 3];
		const double a = a1[i1] - a0[i1];
		const double b = -(a1[i0] - a0[i0]);
		const double c = -a * a0[i0] - b * a0[i1];
		dd[k] = (a * p[i0] + b * p[i1]) + c;
	}
	return (dd[0] * dd[1] > 0.0 && dd[0] * dd[2] > 0.0) ? 1 : 0;
}

static int or_coplanar(const double N[3], const double *V[3], const double *U[3])
{
	const double a0 = fabs(N[0]), a1 = fabs(N[1]), a2 = fabs(N[2]);
	int i0, i1;
	if (a0 > a1) {
		if (a0 > a2) { i0 = 1; i1 = 2; }
		else         { i0 = 0; i1 = 1; }
	} else {
		if (a2 > a1) { i0 = 0; i1 = 1; }
		else         { i0 = 0; i1 = 2; }
	}
	if (or_edge_against_tri(V[0], V[1], U, i0, i1)) return 1;
	if (or_edge_against_tri(V[1], V[2], U, i0, i1)) return 1;
	if (or_edge_against_tri(V[2], V[0], U, i0, i1)) return 1;
	if (or_point_in_tri(V[0], U, i0, i1)) return 1;
	if (or_point_in_tri(U[0], V, i0, i1)) return 1;
	return 0;
}

/* Signed plane distances of the vertices of T to the plane of S (unnormalised),
 * as N.x + d with d = -N.s0; optional snap of |dist| < eps to 0. */
static void or_plane_dists(const double *S[3], const double *T[3], double eps, double N[3], double dist[3])
{
	double e1[3], e2[3];
	or_sub3(S[1], S[0], e1);
	or_sub3(S[2], S[0], e2);
	or_cross3(e1, e2, N);
	const double d = -or_dot3(N, S[0]);
	for (int k = 0; k < 3; k++) {
		double v = or_dot3(N, T[k]) + d;
		if (fabs(v) < eps)
			v = 0.0;
		dist[k] = v;
	}
}

/* Choose the vertex alone on its side of the other plane; returns -1 when all three distances are 0. */
static int or_lone_vertex(const double D[3])
{
	const double d01 = D[0] * D[1], d02 = D[0] * D[2];
	if (d01 > 0.0) return 2;
	if (d02 > 0.0) return 1;
	if (D[1] * D[2] > 0.0 || D[0] != 0.0) return 0;
	if (D[1] != 0.0) return 1;
	if (D[2] != 0.0) return 2;
	return -1;
}

/* The two other vertex indices in the order the published algorithm visits them. */
static void or_others(int lone, int *o1, int *o2)
{
	if (lone == 0) { *o1 = 1; *o2 = 2; }
	else if (lone == 1) { *o1 = 0; *o2 = 2; }
	else { *o1 = 0; *o2 = 1; }
}

/* Interval of a triangle on the intersection line (projection onto axis `ax`):
 * endpoints p_l + (p_o - p_l) * D_l / (D_l - D_o). */
static void or_interval(const double *T[3], const double D[3], int lone, int ax, double out[2])
{
	int o1, o2;
	or_others(lone, &o1, &o2);
	const double pl = T[lone][ax];
	out[0] = pl + ((T[o1][ax] - pl) * D[lone]) / (D[lone] - D[o1]);
	out[1] = pl + ((T[o2][ax] - pl) * D[lone]) / (D[lone] - D[o2]);
}

static int or_max_axis(const double D[3])
{
	double m = fabs(D[0]);
	int idx = 0;
	const double b = fabs(D[1]), c = fabs(D[2]);
	if (b > m) { m = b; idx = 1; }
	if (c > m) { m = c; idx = 2; }
	return idx;
}

/* Boolean test; V = first triangle (env), U = second (robot). */
OR_EXPORT int or_tri_tri(const double *V0, const double *V1, const double *V2,
                         const double *U0, const double *U1, const double *U2, double eps)
{
	const double *V[3] = { V0, V1, V2 };
	const double *U[3] = { U0, U1, U2 };
	double N1[3], N2[3], du[3], dv[3];
	or_plane_dists(V, U, eps, N1, du);
	if (du[0] * du[1] > 0.0 && du[0] * du[2] > 0.0)
		return 0;
	or_plane_dists(U, V, eps, N2, dv);
	if (dv[0] * dv[1] > 0.0 && dv[0] * dv[2] > 0.0)
		return 0;
	double Dl[3];
	or_cross3(N1, N2, Dl);
	const int ax = or_max_axis(Dl);
	const int lv = or_lone_vertex(dv);
	if (lv < 0)
		return or_coplanar(N1, V, U);
	const int lu = or_lone_vertex(du);
	if (lu < 0)
		return or_coplanar(N1, V, U);
	double iv[2], iu[2];
	or_interval(V, dv, lv, ax, iv);
	or_interval(U, du, lu, ax, iu);
	if (iv[0] > iv[1]) { const double c = iv[0]; iv[0] = iv[1]; iv[1] = c; }
	if (iu[0] > iu[1]) { const double c = iu[0]; iu[0] = iu[1]; iu[1] = c; }
	if (iv[1] < iu[0] || iu[1] < iv[0])
		return 0;
	return 1;
}

/* Interval plus the 3-D points where the triangle's edges cross the other plane. */
static void or_interval_pts(const double *T[3], const double D[3], int lone, int ax,
                            double iv[2], double p0[3], double p1[3])
{
	int o1, o2;
	or_others(lone, &o1, &o2);
	const double *A = T[lone];
	const double pl = A[ax];
	double r = D[lone] / (D[lone] - D[o1]);
	iv[0] = pl + (T[o1][ax] - pl) * r;
	for (int c = 0; c < 3; c++) {
		const double diff = (T[o1][c] - A[c]) * r;
		p0[c] = diff + A[c];
	}
	r = D[lone] / (D[lone] - D[o2]);
	iv[1] = pl + (T[o2][ax] - pl) * r;
	for (int c = 0; c < 3; c++) {
		const double diff = (T[o2][c] - A[c]) * r;
		p1[c] = A[c] + diff;
	}
}

/* Test with intersection segment (Moeller 2001 extension).  Returns 1 when the
 * triangles intersect.  On a coplanar pair *coplanar = 1 and the points are
 * zero; on a miss the points are zero. */
OR_EXPORT int or_tri_tri_isect(const double *V0, const double *V1, const double *V2,
                               const double *U0, const double *U1, const double *U2, double eps,
                               int *coplanar, double pt1[3], double pt2[3])
{
	const double *V[3] = { V0, V1, V2 };
	const double *U[3] = { U0, U1, U2 };
	double N1[3], N2[3], du[3], dv[3];
	*coplanar = 0;
	for (int c = 0; c < 3; c++) { pt1[c] = 0.0; pt2[c] = 0.0; }
	or_plane_dists(V, U, eps, N1, du);
	if (du[0] * du[1] > 0.0 && du[0] * du[2] > 0.0)
		return 0;
	or_plane_dists(U, V, eps, N2, dv);
	if (dv[0] * dv[1] > 0.0 && dv[0] * dv[2] > 0.0)
		return 0;
	double Dl[3];
	or_cross3(N1, N2, Dl);
	const int ax = or_max_axis(Dl);
	const int lv = or_lone_vertex(dv);
	if (lv < 0) {
		*coplanar = 1;
		return or_coplanar(N1, V, U);
	}
	const int lu = or_lone_vertex(du);
	if (lu < 0) {
		*coplanar = 1;
		return or_coplanar(N1, V, U);
	}
	double iv[2], iu[2], a1[3], a2[3], b1[3], b2[3];
	or_interval_pts(V, dv, lv, ax, iv, a1, a2);
	or_interval_pts(U, du, lu, ax, iu, b1, b2);
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

/* ------------------------------------------------------------------------ */
/* Oriented-box overlap (separating-axis theorem, Gottschalk et al. 1996)    */
/* ------------------------------------------------------------------------ */

/* Box A: axis-aligned, half-extents ea.  Box B: axes = columns of R, half
 * extents eb, centre offset T = cB - cA.  AR = |R| + slack.  Returns 1 when a
 * separating axis exists (strict inequality, touching counts as overlap). */
static int or_sat_disjoint(const double ea[3], const double eb[3], const double T[3],
                           const double R[9], const double AR[9])
{
#define RR(i, j) R[3 * (i) + (j)]
#define AA(i, j) AR[3 * (i) + (j)]
	for (int i = 0; i < 3; i++) {
		const double rb = (eb[0] * AA(i, 0) + eb[1] * AA(i, 1)) + eb[2] * AA(i, 2);
		if (fabs(T[i]) > ea[i] + rb) return 1;
	}
	for (int j = 0; j < 3; j++) {
		const double tl = (T[0] * RR(0, j) + T[1] * RR(1, j)) + T[2] * RR(2, j);
		const double ra = (ea[0] * AA(0, j) + ea[1] * AA(1, j)) + ea[2] * AA(2, j);
		if (fabs(tl) > ra + eb[j]) return 1;
	}
	for (int i = 0; i < 3; i++) {
		const int i1 = (i + 1) % 3, i2 = (i + 2) % 3;
		for (int j = 0; j < 3; j++) {
			const int j1 = (j + 1) % 3, j2 = (j + 2) % 3;
			const double tl = T[i2] * RR(i1, j) - T[i1] * RR(i2, j);
			const double ra = ea[i1] * AA(i2, j) + ea[i2] * AA(i1, j);
			const double rb = eb[j1] * AA(i, j2) + eb[j2] * AA(i, j1);
			if (fabs(tl) > ra + rb) return 1;
		}
	}
	return 0;
#undef RR
#undef AA
}

/* ------------------------------------------------------------------------ */
/* Meshes, the unit-world recipe and a CPU BVH                               */
/* ------------------------------------------------------------------------ */

typedef struct {
	double lo[3], hi[3];
	int left, right;   /* children, -1 for a leaf */
	int first, count;  /* leaf triangle range in `order` */
	/* oriented box: axes as rows of E (orthonormal), centre c, half-extents h */
	double E[9], c[3], h[3];
} or_node;

typedef struct {
	int64_t nv, nf;
	double *V;     /* CD vertices (nv x 3): env in world frame, robot in its local frame */
	int32_t *F;    /* faces (nf x 3) */
	int32_t *order;
	or_node *nodes;
	int nnodes;
	double aabb_lo[3], aabb_hi[3];
	double rmax;   /* max |vertex| (inf-norm rows, summed) for the box margin */
} or_mesh;

typedef struct or_world {
	or_mesh env, rob;
	double *env_local; /* env CD vertices before the perturbation transform */
	float scale;
	float center[3];
	float ompl_center[3]; /* float mean of the robot's vertices (scene.cc:40-50,141-145) */
	double pert[7];
	double env_box_c[3], env_box_h[3]; /* local AABB box of the env CD model */
	double rob_box_c[3], rob_box_h[3];
	double pert_R[9], pert_t[3];
} or_world;

static void or_mesh_free(or_mesh *m)
{
	free(m->V); free(m->F); free(m->order); free(m->nodes);
	memset(m, 0, sizeof(*m));
}

static const double *or_tri_vertex(const or_mesh *m, int64_t tri, int k)
{
	return m->V + 3 * (int64_t)m->F[3 * tri + k];
}

/* Eigenvectors (rows of E) of the symmetric matrix S = (xx, yy, zz, xy, xz, yz):
 * cyclic Jacobi rotations (Golub and Van Loan, section 8.5), then Gram-Schmidt
 * and a cross product so that E is orthonormal to rounding. */
static void or_eigen3(const double S[6], double E[9])
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
				const double c = 1.0 / sqrt(t * t + 1.0), sn = t * c;
				for (int k = 0; k < 3; k++) {
					const double x = a[k][p], y = a[k][q];
					a[k][p] = c * x - sn * y;
					a[k][q] = sn * x + c * y;
				}
				for (int k = 0; k < 3; k++) {
					const double x = a[p][k], y = a[q][k];
					a[p][k] = c * x - sn * y;
					a[q][k] = sn * x + c * y;
				}
				for (int k = 0; k < 3; k++) {
					const double x = v[k][p], y = v[k][q];
					v[k][p] = c * x - sn * y;
					v[k][q] = sn * x + c * y;
				}
			}
	}
	double e0[3] = { v[0][0], v[1][0], v[2][0] }, e1[3] = { v[0][1], v[1][1], v[2][1] };
	const double n0 = sqrt(e0[0] * e0[0] + e0[1] * e0[1] + e0[2] * e0[2]);
	for (int k = 0; k < 3; k++) e0[k] /= n0;
	const double d = e0[0] * e1[0] + e0[1] * e1[1] + e0[2] * e1[2];
	for (int k = 0; k < 3; k++) e1[k] -= d * e0[k];
	const double n1 = sqrt(e1[0] * e1[0] + e1[1] * e1[1] + e1[2] * e1[2]);
	for (int k = 0; k < 3; k++) e1[k] /= n1;
	E[0] = e0[0]; E[1] = e0[1]; E[2] = e0[2];
	E[3] = e1[0]; E[4] = e1[1]; E[5] = e1[2];
	E[6] = e0[1] * e1[2] - e0[2] * e1[1];
	E[7] = e0[2] * e1[0] - e0[0] * e1[2];
	E[8] = e0[0] * e1[1] - e0[1] * e1[0];
}

/* Oriented box of the node's triangles: principal axes of their vertices, the
 * projections' range, extents widened by 1e-12 of the coordinates (the FP64
 * projections' rounding). */
static void or_fit_obb(const or_mesh *m, or_node *n)
{
	double mu[3] = { 0, 0, 0 }, S[6] = { 0, 0, 0, 0, 0, 0 };
	const double cnt = 3.0 * n->count;
	for (int i = n->first; i < n->first + n->count; i++)
		for (int k = 0; k < 3; k++) {
			const double *p = or_tri_vertex(m, m->order[i], k);
			for (int c = 0; c < 3; c++) mu[c] += p[c] / cnt;
		}
	for (int i = n->first; i < n->first + n->count; i++)
		for (int k = 0; k < 3; k++) {
			const double *p = or_tri_vertex(m, m->order[i], k);
			const double d0 = p[0] - mu[0], d1 = p[1] - mu[1], d2 = p[2] - mu[2];
			S[0] += d0 * d0; S[1] += d1 * d1; S[2] += d2 * d2;
			S[3] += d0 * d1; S[4] += d0 * d2; S[5] += d1 * d2;
		}
	or_eigen3(S, n->E);
	double lo[3] = { INFINITY, INFINITY, INFINITY }, hi[3] = { -INFINITY, -INFINITY, -INFINITY }, big = 0.0;
	for (int i = n->first; i < n->first + n->count; i++)
		for (int k = 0; k < 3; k++) {
			const double *p = or_tri_vertex(m, m->order[i], k);
			const double l1 = fabs(p[0]) + fabs(p[1]) + fabs(p[2]);
			if (l1 > big) big = l1;
			for (int a = 0; a < 3; a++) {
				const double pr = n->E[3 * a] * p[0] + n->E[3 * a + 1] * p[1] + n->E[3 * a + 2] * p[2];
				if (pr < lo[a]) lo[a] = pr;
				if (pr > hi[a]) hi[a] = pr;
			}
		}
	for (int k = 0; k < 3; k++) n->c[k] = 0.0;
	for (int a = 0; a < 3; a++) {
		const double mid = 0.5 * (lo[a] + hi[a]);
		n->h[a] = 0.5 * (hi[a] - lo[a]) + 1e-12 * (1.0 + big);
		for (int k = 0; k < 3; k++) n->c[k] += n->E[3 * a + k] * mid;
	}
}

static int or_build_node(or_mesh *m, double *cent, int first, int count, int *next)
{
	const int id = (*next)++;
	or_node *n = &m->nodes[id];
	for (int c = 0; c < 3; c++) { n->lo[c] = INFINITY; n->hi[c] = -INFINITY; }
	double clo[3] = { INFINITY, INFINITY, INFINITY }, chi[3] = { -INFINITY, -INFINITY, -INFINITY };
	for (int i = first; i < first + count; i++) {
		const int t = m->order[i];
		for (int k = 0; k < 3; k++) {
			const double *p = or_tri_vertex(m, t, k);
			for (int c = 0; c < 3; c++) {
				if (p[c] < n->lo[c]) n->lo[c] = p[c];
				if (p[c] > n->hi[c]) n->hi[c] = p[c];
			}
		}
		for (int c = 0; c < 3; c++) {
			if (cent[3 * t + c] < clo[c]) clo[c] = cent[3 * t + c];
			if (cent[3 * t + c] > chi[c]) chi[c] = cent[3 * t + c];
		}
	}
	n->first = first; n->count = count; n->left = n->right = -1;
	or_fit_obb(m, n);
	if (count <= 4)
		return id;
	int axis = 0;
	double ext = chi[0] - clo[0];
	for (int c = 1; c < 3; c++)
		if (chi[c] - clo[c] > ext) { ext = chi[c] - clo[c]; axis = c; }
	if (!(ext > 0.0))
		return id;
	/* partition about the centroid-bounds midpoint; fall back to a count split */
	const double mid = 0.5 * (clo[axis] + chi[axis]);
	int i = first, j = first + count - 1;
	while (i <= j) {
		if (cent[3 * m->order[i] + axis] < mid) i++;
		else { const int t = m->order[i]; m->order[i] = m->order[j]; m->order[j] = t; j--; }
	}
	int nl = i - first;
	if (nl == 0 || nl == count)
		nl = count / 2;
	const int l = or_build_node(m, cent, first, nl, next);
	const int r = or_build_node(m, cent, first + nl, count - nl, next);
	n = &m->nodes[id];
	n->left = l; n->right = r; n->count = 0;
	return id;
}

static void or_mesh_finish(or_mesh *m)
{
	const int64_t nf = m->nf;
	m->order = (int32_t *)malloc(sizeof(int32_t) * (size_t)(nf > 0 ? nf : 1));
	m->nodes = (or_node *)malloc(sizeof(or_node) * (size_t)(2 * nf + 1));
	double *cent = (double *)malloc(sizeof(double) * 3 * (size_t)(nf > 0 ? nf : 1));
	for (int64_t t = 0; t < nf; t++) {
		m->order[t] = (int32_t)t;
		for (int c = 0; c < 3; c++)
			cent[3 * t + c] = (or_tri_vertex(m, t, 0)[c] + or_tri_vertex(m, t, 1)[c] + or_tri_vertex(m, t, 2)[c]) / 3.0;
	}
	int next = 0;
	if (nf > 0)
		or_build_node(m, cent, 0, (int)nf, &next);
	m->nnodes = next;
	free(cent);
	m->rmax = 0.0;
	for (int c = 0; c < 3; c++) { m->aabb_lo[c] = INFINITY; m->aabb_hi[c] = -INFINITY; }
	for (int64_t v = 0; v < m->nv; v++) {
		const double *p = m->V + 3 * v;
		const double r = fabs(p[0]) + fabs(p[1]) + fabs(p[2]);
		if (r > m->rmax) m->rmax = r;
		for (int c = 0; c < 3; c++) {
			if (p[c] < m->aabb_lo[c]) m->aabb_lo[c] = p[c];
			if (p[c] > m->aabb_hi[c]) m->aabb_hi[c] = p[c];
		}
	}
}

OR_EXPORT or_world *or_world_new(void)
{
	or_world *w = (or_world *)calloc(1, sizeof(or_world));
	w->pert[3] = 1.0;
	const double q[7] = { 0, 0, 0, 1, 0, 0, 0 };
	or_state_transform(q, w->pert_R, w->pert_t);
	return w;
}

OR_EXPORT void or_world_free(or_world *w)
{
	if (!w) return;
	or_mesh_free(&w->env);
	or_mesh_free(&w->rob);
	free(w->env_local);
	free(w);
}

/* Bounding box seeded at the origin, extended with every vertex (bbox.h:21-51); float. */
static float or_span(const float *V, int64_t nv)
{
	float lo[3] = { 0.f, 0.f, 0.f }, hi[3] = { 0.f, 0.f, 0.f };
	for (int64_t i = 0; i < nv; i++)
		for (int c = 0; c < 3; c++) {
			const float x = V[3 * i + c];
			if (x > hi[c]) hi[c] = x;
			if (x < lo[c]) lo[c] = x;
		}
	float s = hi[0] - lo[0];
	const float sy = hi[1] - lo[1], sz = hi[2] - lo[2];
	if (sy > s) s = sy;
	if (sz > s) s = sz;
	return s;
}

static void or_local_aabb_box(const or_mesh *m, double c[3], double h[3])
{
	for (int k = 0; k < 3; k++) {
		c[k] = (m->aabb_lo[k] + m->aabb_hi[k]) * 0.5;
		h[k] = (m->aabb_hi[k] - m->aabb_lo[k]) * 0.5;
	}
}

static void or_apply_env_transform(or_world *w)
{
	for (int64_t v = 0; v < w->env.nv; v++)
		or_xform_point(w->pert_R, w->pert_t, w->env_local + 3 * v, w->env.V + 3 * v);
	free(w->env.order); free(w->env.nodes);
	w->env.order = NULL; w->env.nodes = NULL;
	or_mesh_finish(&w->env);
}

/*
 * load + scaleToUnit + angleModel(0, 0) (unit_world.cc:94-161, scene.cc:78-229, cdmodel.cc:120-160).
 * centre == NULL: robot centre = float mean of its vertices (scene.cc:141-145);
 * otherwise the enforced centre (unit_world.cc:114-118).
 */
OR_EXPORT int or_world_set_meshes(or_world *w,
                                  const float *Ve, int64_t nve, const uint32_t *Fe, int64_t nfe,
                                  const float *Vr, int64_t nvr, const uint32_t *Fr, int64_t nfr,
                                  const float *center)
{
	or_mesh_free(&w->env);
	or_mesh_free(&w->rob);
	free(w->env_local);
	w->env_local = NULL;
	const float span_e = or_span(Ve, nve);
	const float span_r = or_span(Vr, nvr);
	const float mx = span_e > span_r ? span_e : span_r;
	w->scale = (float)(1.0 / (double)mx);
	{
		float acc[3] = { 0.f, 0.f, 0.f };
		for (int64_t i = 0; i < nvr; i++)
			for (int c = 0; c < 3; c++) acc[c] = acc[c] + Vr[3 * i + c];
		for (int c = 0; c < 3; c++) w->ompl_center[c] = nvr > 0 ? acc[c] / (float)nvr : 0.0f;
	}
	for (int c = 0; c < 3; c++) w->center[c] = center ? center[c] : w->ompl_center[c];
	const double s = (double)w->scale;
	/* robot xform = S(s) T(-c) in float: translation column fl32(s * -c) */
	float tr[3];
	for (int c = 0; c < 3; c++) tr[c] = w->scale * (-w->center[c]);
	w->env.nv = nve; w->env.nf = nfe;
	w->env.V = (double *)malloc(sizeof(double) * 3 * (size_t)(nve > 0 ? nve : 1));
	w->env_local = (double *)malloc(sizeof(double) * 3 * (size_t)(nve > 0 ? nve : 1));
	w->env.F = (int32_t *)malloc(sizeof(int32_t) * 3 * (size_t)(nfe > 0 ? nfe : 1));
	for (int64_t i = 0; i < 3 * nve; i++)
		w->env_local[i] = s * (double)Ve[i];
	for (int64_t i = 0; i < 3 * nfe; i++)
		w->env.F[i] = (int32_t)Fe[i];
	w->rob.nv = nvr; w->rob.nf = nfr;
	w->rob.V = (double *)malloc(sizeof(double) * 3 * (size_t)(nvr > 0 ? nvr : 1));
	w->rob.F = (int32_t *)malloc(sizeof(int32_t) * 3 * (size_t)(nfr > 0 ? nfr : 1));
	for (int64_t i = 0; i < nvr; i++)
		for (int c = 0; c < 3; c++)
			w->rob.V[3 * i + c] = s * (double)Vr[3 * i + c] + (double)tr[c];
	for (int64_t i = 0; i < 3 * nfr; i++)
		w->rob.F[i] = (int32_t)Fr[i];
	/* local boxes for isDisentangled come from the untransformed CD vertices */
	{
		or_mesh tmp;
		memset(&tmp, 0, sizeof(tmp));
		tmp.nv = nve; tmp.V = w->env_local;
		for (int c = 0; c < 3; c++) { tmp.aabb_lo[c] = INFINITY; tmp.aabb_hi[c] = -INFINITY; }
		for (int64_t v = 0; v < nve; v++)
			for (int c = 0; c < 3; c++) {
				const double x = w->env_local[3 * v + c];
				if (x < tmp.aabb_lo[c]) tmp.aabb_lo[c] = x;
				if (x > tmp.aabb_hi[c]) tmp.aabb_hi[c] = x;
			}
		or_local_aabb_box(&tmp, w->env_box_c, w->env_box_h);
	}
	or_apply_env_transform(w);
	or_mesh_finish(&w->rob);
	or_local_aabb_box(&w->rob, w->rob_box_c, w->rob_box_h);
	return 0;
}

/* set_perturbation (unit_world.cc:164-168): the env CD model is placed by this state. */
OR_EXPORT int or_world_set_perturbation(or_world *w, const double q[7])
{
	memcpy(w->pert, q, sizeof(double) * 7);
	or_state_transform(q, w->pert_R, w->pert_t);
	if (w->env_local)
		or_apply_env_transform(w);
	return 0;
}

/* info: [scale, cx, cy, cz, nv_env, nf_env, nv_rob, nf_rob] */
OR_EXPORT void or_world_info(const or_world *w, double *out)
{
	out[0] = (double)w->scale;
	out[1] = w->center[0]; out[2] = w->center[1]; out[3] = w->center[2];
	out[4] = (double)w->env.nv; out[5] = (double)w->env.nf;
	out[6] = (double)w->rob.nv; out[7] = (double)w->rob.nf;
}

/* which = 0: env world-frame CD vertices; 1: robot local CD vertices. */
OR_EXPORT void or_world_vertices(const or_world *w, int which, double *out)
{
	const or_mesh *m = which ? &w->rob : &w->env;
	memcpy(out, m->V, sizeof(double) * 3 * (size_t)m->nv);
}

/* ------------------------------------------------------------------------ */
/* Queries                                                                   */
/* ------------------------------------------------------------------------ */

typedef struct {
	double R[9], t[3], AR[9];
	double margin, slack;
	const or_world *w;
	/* collection for intersecting_segments */
	int collect;
	int64_t cap, count;
	int32_t *pairs;
} or_query;

static void or_query_init(or_query *qq, const or_world *w, const double q[7])
{
	or_state_transform(q, qq->R, qq->t);
	const double s = ((q[4] * q[4] + q[5] * q[5]) + q[6] * q[6]) + q[3] * q[3];
	const double dev = fabs(1.0 - s);
	const double slack = 1e-12 + 2.0 * dev;
	for (int i = 0; i < 9; i++) qq->AR[i] = fabs(qq->R[i]) + slack;
	qq->slack = 3.0 * slack;   /* |M| = |Ea R Eb^T|: the rotation's slack through two unit-row products */
	const double W = fabs(q[0]) + fabs(q[1]) + fabs(q[2]) + w->rob.rmax + w->env.rmax;
	qq->margin = 1e-12 * (1.0 + W) + 8.0 * dev * W;
	qq->w = w;
	qq->collect = 0;
	qq->cap = qq->count = 0;
	qq->pairs = NULL;
}

/* The two nodes' oriented boxes (as FCL's OBBRSS nodes are, cdmodel.cc:17-18):
 * the robot box brought into the env box's frame, M = Ea R Eb^T and
 * T = Ea (R cb + t - ca), then the separating-axis test with the query's slack
 * on |M| and margins on the extents. */
static int or_nodes_disjoint(const or_query *qq, const or_node *a, const or_node *b)
{
	double ea[3], eb[3], CB[3], d[3], T[3], N[9], M[9], AM[9];
	for (int c = 0; c < 3; c++) {
		ea[c] = a->h[c] + qq->margin;
		eb[c] = b->h[c] + qq->margin;
	}
	or_xform_point(qq->R, qq->t, b->c, CB);
	for (int c = 0; c < 3; c++) d[c] = CB[c] - a->c[c];
	for (int i = 0; i < 3; i++)
		T[i] = (a->E[3 * i] * d[0] + a->E[3 * i + 1] * d[1]) + a->E[3 * i + 2] * d[2];
	/* column j of N: robot box axis j in the env frame (R times row j of Eb) */
	for (int i = 0; i < 3; i++)
		for (int j = 0; j < 3; j++)
			N[3 * i + j] = (qq->R[3 * i] * b->E[3 * j] + qq->R[3 * i + 1] * b->E[3 * j + 1]) +
			               qq->R[3 * i + 2] * b->E[3 * j + 2];
	for (int i = 0; i < 3; i++)
		for (int j = 0; j < 3; j++) {
			M[3 * i + j] = (a->E[3 * i] * N[j] + a->E[3 * i + 1] * N[3 + j]) + a->E[3 * i + 2] * N[6 + j];
			AM[3 * i + j] = fabs(M[3 * i + j]) + qq->slack;
		}
	return or_sat_disjoint(ea, eb, T, M, AM);
}

/* Leaf-leaf: Moeller (eps 0) on every triangle pair.  Returns 1 on the first hit
 * unless collecting, in which case every hit pair is recorded. */
static int or_leaf_pair(or_query *qq, const or_node *a, const or_node *b)
{
	const or_world *w = qq->w;
	int hit = 0;
	for (int j = b->first; j < b->first + b->count; j++) {
		const int rt = w->rob.order[j];
		double U[3][3];
		for (int k = 0; k < 3; k++)
			or_xform_point(qq->R, qq->t, or_tri_vertex(&w->rob, rt, k), U[k]);
		for (int i = a->first; i < a->first + a->count; i++) {
			const int et = w->env.order[i];
			if (or_tri_tri(or_tri_vertex(&w->env, et, 0), or_tri_vertex(&w->env, et, 1),
			               or_tri_vertex(&w->env, et, 2), U[0], U[1], U[2], 0.0)) {
				if (!qq->collect)
					return 1;
				if (qq->count < qq->cap) {
					qq->pairs[2 * qq->count + 0] = et;
					qq->pairs[2 * qq->count + 1] = rt;
				}
				qq->count++;
				hit = 1;
			}
		}
	}
	return hit;
}

static int or_traverse(or_query *qq)
{
	const or_world *w = qq->w;
	if (w->env.nnodes == 0 || w->rob.nnodes == 0)
		return 0;
	int cap = 256, top = 0;
	int *stack = (int *)malloc(sizeof(int) * 2 * (size_t)cap);
	stack[top++] = 0; stack[top++] = 0;
	int hit = 0;
	while (top > 0) {
		const int bi = stack[--top];
		const int ai = stack[--top];
		const or_node *a = &w->env.nodes[ai];
		const or_node *b = &w->rob.nodes[bi];
		if (or_nodes_disjoint(qq, a, b))
			continue;
		const int la = a->left < 0, lb = b->left < 0;
		if (la && lb) {
			if (or_leaf_pair(qq, a, b)) {
				hit = 1;
				if (!qq->collect) break;
			}
			continue;
		}
		if (top + 4 > 2 * cap) {
			cap *= 2;
			stack = (int *)realloc(stack, sizeof(int) * 2 * (size_t)cap);
		}
		double sa = 0, sb = 0;
		for (int c = 0; c < 3; c++) { sa += a->h[c]; sb += b->h[c]; }
		if (!la && (lb || sa >= sb)) {
			stack[top++] = a->right; stack[top++] = bi;
			stack[top++] = a->left;  stack[top++] = bi;
		} else {
			stack[top++] = ai; stack[top++] = b->right;
			stack[top++] = ai; stack[top++] = b->left;
		}
	}
	free(stack);
	return hit;
}

/* Brute force over all triangle pairs (small meshes; the BVH cross-check). */
static int or_collide_brute(const or_world *w, const double q[7])
{
	double R[9], t[3];
	or_state_transform(q, R, t);
	for (int64_t r = 0; r < w->rob.nf; r++) {
		double U[3][3];
		for (int k = 0; k < 3; k++)
			or_xform_point(R, t, or_tri_vertex(&w->rob, r, k), U[k]);
		for (int64_t e = 0; e < w->env.nf; e++)
			if (or_tri_tri(or_tri_vertex(&w->env, e, 0), or_tri_vertex(&w->env, e, 1),
			               or_tri_vertex(&w->env, e, 2), U[0], U[1], U[2], 0.0))
				return 1;
	}
	return 0;
}

/* isValid (unit_world.cc:215-247): true when no triangle pair intersects;
 * true as well when a model is missing. */
OR_EXPORT int or_is_valid(const or_world *w, const double q[7], int brute)
{
	if (w->env.nf == 0 || w->rob.nf == 0)
		return 1;
	if (brute)
		return !or_collide_brute(w, q);
	or_query qq;
	or_query_init(&qq, w, q);
	return !or_traverse(&qq);
}

/* isDisentangled (unit_world.cc:249-264, cdmodel.cc:180-197): the robot's local
 * AABB box placed by robTf * uncentrializer against the env's, placed by envTf. */
OR_EXPORT int or_is_disentangled(const or_world *w, const double q[7])
{
	double R[9], t[3];
	or_state_transform(q, R, t);
	const double *Re = w->pert_R, *te = w->pert_t;
	double cr[3], ce[3];
	or_xform_point(R, t, w->rob_box_c, cr);
	or_xform_point(Re, te, w->env_box_c, ce);
	/* express the robot box in the env box frame: Rr = Re^T R, T = Re^T (cr - ce) */
	double Rr[9], T[3], AR[9], d[3];
	for (int c = 0; c < 3; c++) d[c] = cr[c] - ce[c];
	for (int i = 0; i < 3; i++) {
		T[i] = (Re[0 * 3 + i] * d[0] + Re[1 * 3 + i] * d[1]) + Re[2 * 3 + i] * d[2];
		for (int j = 0; j < 3; j++)
			Rr[3 * i + j] = (Re[0 * 3 + i] * R[0 * 3 + j] + Re[1 * 3 + i] * R[1 * 3 + j]) + Re[2 * 3 + i] * R[2 * 3 + j];
	}
	for (int i = 0; i < 9; i++) AR[i] = fabs(Rr[i]);
	return or_sat_disjoint(w->env_box_h, w->rob_box_h, T, Rr, AR);
}

/*
 * transitStateToWithContact (unit_world.cc:405-474).  Returns the number of
 * isValid calls made.  first_step: index of the first colliding step (0-based),
 * -1 when every step is free (done), -2 when no step was taken (delta >= dist).
 * last_free / state / last_tau / tau follow the reference's tuple, including
 * its outer `tau` staying 0 when the loop completes.
 */
OR_EXPORT int64_t or_transit_with_contact(const or_world *w, const double from[7], const double to[7],
                                          double verify_delta, double *last_free, double *state,
                                          int *done, float *last_tau_out, float *tau_out,
                                          int64_t *first_step)
{
	const double dist = or_distance(from, to);
	memcpy(last_free, from, sizeof(double) * 7);
	if (!(verify_delta >= dist) && dist == dist &&
	    (!(verify_delta > 0.0) || dist / verify_delta > 1073741824.0)) {
		/* the reference loop never ends for delta <= 0; the step cap keeps it finite */
		memcpy(state, from, sizeof(double) * 7);
		*done = 0; *last_tau_out = 0.0f; *tau_out = 0.0f;
		*first_step = -3;
		return 0;
	}
	if (verify_delta >= dist || !(dist == dist)) {
		memcpy(state, to, sizeof(double) * 7);
		*done = 0; *last_tau_out = 0.0f; *tau_out = 1.0f;
		*first_step = -2;
		if (!(dist == dist)) {
			/* the reference's loop is skipped entirely for a NaN distance */
			memcpy(state, from, sizeof(double) * 7);
			*tau_out = 0.0f;
		}
		return 0;
	}
	double delta = verify_delta;
	const double inv_dist = 1.0 / dist;
	double last_tau = 0.0;
	int64_t k = 0;
	memcpy(state, from, sizeof(double) * 7);
	while (delta <= dist) {
		const double tau = delta * inv_dist;
		or_interpolate(from, to, tau, state);
		if (!or_is_valid(w, state, 0)) {
			*done = 0; *last_tau_out = (float)last_tau; *tau_out = (float)tau;
			*first_step = k;
			return k + 1;
		}
		last_tau = tau;
		memcpy(last_free, state, sizeof(double) * 7);
		if (delta < dist) {
			delta = delta + verify_delta;
			delta = dist < delta ? dist : delta;
		} else {
			delta = delta + verify_delta;
		}
		k++;
	}
	*done = delta > dist;
	*last_tau_out = (float)last_tau;
	*tau_out = 0.0f;
	*first_step = -1;
	return k;
}

/* isValidTransition (unit_world.cc:477-486) uses delta' = min(dist / 2, delta). */
static double or_transition_delta(const double a[7], const double b[7], double delta)
{
	const double d = or_distance(a, b);
	const double h = d / 2.0;
	return h < delta ? h : delta;
}

OR_EXPORT void or_states_valid(const or_world *w, const double *q, int64_t n, uint8_t *out, int nthreads)
{
#ifdef _OPENMP
	if (nthreads > 0) omp_set_num_threads(nthreads);
#pragma omp parallel for schedule(dynamic, 16)
#endif
	for (int64_t i = 0; i < n; i++)
		out[i] = (uint8_t)or_is_valid(w, q + 7 * i, 0);
	(void)nthreads;
}

OR_EXPORT void or_states_valid_brute(const or_world *w, const double *q, int64_t n, uint8_t *out, int nthreads)
{
#ifdef _OPENMP
	if (nthreads > 0) omp_set_num_threads(nthreads);
#pragma omp parallel for schedule(dynamic, 4)
#endif
	for (int64_t i = 0; i < n; i++)
		out[i] = (uint8_t)or_is_valid(w, q + 7 * i, 1);
	(void)nthreads;
}

OR_EXPORT void or_states_disentangled(const or_world *w, const double *q, int64_t n, uint8_t *out, int nthreads)
{
#ifdef _OPENMP
	if (nthreads > 0) omp_set_num_threads(nthreads);
#pragma omp parallel for schedule(static)
#endif
	for (int64_t i = 0; i < n; i++)
		out[i] = (uint8_t)or_is_disentangled(w, q + 7 * i);
	(void)nthreads;
}

/* Batched segments.  mode 0: transit_state_to(delta); mode 1: is_valid_transition(delta).
 * out_first gets the first-contact step (see or_transit_with_contact); out_checks the isValid count. */
OR_EXPORT void or_segments_first_contact(const or_world *w, const double *q0, const double *q1, int64_t n,
                                         double delta, int mode, int32_t *out_first, int64_t *out_checks,
                                         int nthreads)
{
#ifdef _OPENMP
	if (nthreads > 0) omp_set_num_threads(nthreads);
#pragma omp parallel for schedule(dynamic, 1)
#endif
	for (int64_t i = 0; i < n; i++) {
		const double *a = q0 + 7 * i, *b = q1 + 7 * i;
		const double d = mode ? or_transition_delta(a, b, delta) : delta;
		double lf[7], st[7];
		int done;
		float lt, tt;
		int64_t first;
		const int64_t checks = or_transit_with_contact(w, a, b, d, lf, st, &done, &lt, &tt, &first);
		out_first[i] = (int32_t)first;
		if (out_checks) out_checks[i] = checks;
	}
	(void)nthreads;
}

/* Number of steps the reference loop takes for one segment (no collision checks). */
OR_EXPORT int64_t or_segment_steps(const double from[7], const double to[7], double verify_delta)
{
	const double dist = or_distance(from, to);
	if (verify_delta >= dist || !(dist == dist))
		return 0;
	if (!(verify_delta > 0.0) || dist / verify_delta > 1073741824.0)
		return -1;
	double delta = verify_delta;
	int64_t k = 0;
	while (delta <= dist) {
		if (delta < dist) {
			delta = delta + verify_delta;
			delta = dist < delta ? dist : delta;
		} else {
			delta = delta + verify_delta;
		}
		k++;
	}
	return k;
}

/* State at step k of a segment (the k-th state the reference loop checks). */
OR_EXPORT void or_segment_state(const double from[7], const double to[7], double verify_delta, int64_t k,
                                double out[7], double *tau_out)
{
	const double dist = or_distance(from, to);
	const double inv_dist = 1.0 / dist;
	double delta = verify_delta;
	for (int64_t j = 0; j < k; j++) {
		if (delta < dist) {
			delta = delta + verify_delta;
			delta = dist < delta ? dist : delta;
		} else {
			delta = delta + verify_delta;
		}
	}
	const double tau = delta * inv_dist;
	or_interpolate(from, to, tau, out);
	*tau_out = tau;
}

static int or_cmp_pair(const void *a, const void *b)
{
	const int32_t *x = (const int32_t *)a, *y = (const int32_t *)b;
	if (x[0] != y[0]) return x[0] < y[0] ? -1 : 1;
	if (x[1] != y[1]) return x[1] < y[1] ? -1 : 1;
	return 0;
}

/*
 * intersectingSegments (unit_world.cc:959-1012): every (env, robot) face pair
 * the collision predicate reports, sorted by (env, robot), each with Moeller's
 * intersection segment at the reference's 1e-6 snap.  Returns the pair count
 * (outputs are filled up to `cap`).  coplanar/missed pairs get zero points.
 */
OR_EXPORT int64_t or_intersecting_segments(const or_world *w, const double q[7], int64_t cap,
                                           double *begins, double *ends, double *mags,
                                           int32_t *pairs, int32_t *coplanar)
{
	or_query qq;
	or_query_init(&qq, w, q);
	qq.collect = 1;
	int64_t tmpcap = 1024;
	qq.cap = tmpcap;
	qq.pairs = (int32_t *)malloc(sizeof(int32_t) * 2 * (size_t)tmpcap);
	or_traverse(&qq);
	if (qq.count > tmpcap) {
		free(qq.pairs);
		tmpcap = qq.count;
		or_query_init(&qq, w, q);
		qq.collect = 1;
		qq.cap = tmpcap;
		qq.pairs = (int32_t *)malloc(sizeof(int32_t) * 2 * (size_t)tmpcap);
		or_traverse(&qq);
	}
	const int64_t m = qq.count;
	qsort(qq.pairs, (size_t)m, sizeof(int32_t) * 2, or_cmp_pair);
	for (int64_t i = 0; i < m && i < cap; i++) {
		const int et = qq.pairs[2 * i], rt = qq.pairs[2 * i + 1];
		double U[3][3];
		for (int k = 0; k < 3; k++)
			or_xform_point(qq.R, qq.t, or_tri_vertex(&w->rob, rt, k), U[k]);
		int cop = 0;
		double p1[3], p2[3];
		or_tri_tri_isect(or_tri_vertex(&w->env, et, 0), or_tri_vertex(&w->env, et, 1),
		                 or_tri_vertex(&w->env, et, 2), U[0], U[1], U[2], 1e-6, &cop, p1, p2);
		for (int c = 0; c < 3; c++) { begins[3 * i + c] = p1[c]; ends[3 * i + c] = p2[c]; }
		const double dx = p2[0] - p1[0], dy = p2[1] - p1[1], dz = p2[2] - p1[2];
		mags[i] = sqrt((dx * dx + dy * dy) + dz * dz);
		pairs[2 * i] = et; pairs[2 * i + 1] = rt;
		if (coplanar) coplanar[i] = cop;
	}
	free(qq.pairs);
	return m;
}

/* ------------------------------------------------------------------------ */
/* OMPL's discrete motion check over OMPL.app's SE3StateSpace, the check    */
/* behind OmplDriver::validateMotionPairs (lib/pyse3ompl/ompldriver.cc:     */
/* 597-621, resolution set at :676-677).  OMPL is not vendored by the       */
/* reference (a fork of OMPL 1.x); this restates its published algorithm:   */
/* SpaceInformation::setStateValidityCheckingResolution sets each           */
/* component's longest valid segment to extent * fraction (R^3 extent       */
/* |hi - lo|, SO(3) extent pi/2); the compound validSegmentCount is the     */
/* largest component count ceil(d / lvs) (R^3 Euclidean distance, SO(3) arc */
/* length acos|<q1,q2>|, 0 above 1 - 1e-9); DiscreteMotionValidator checks  */
/* s2 and interpolate(s1, s2, k / nd) for k = 1 .. nd - 1, not s1.          */
/* OMPL states are (x, y, z, qx, qy, qz, qw).                               */
/* ------------------------------------------------------------------------ */

static double or_ompl_dot(const double *a, const double *b)
{
	return ((a[3] * b[3] + a[4] * b[4]) + a[5] * b[5]) + a[6] * b[6];
}

static double or_ompl_arc(double dq)
{
	const double a = fabs(dq);
	return a > 1.0 - 1e-9 ? 0.0 : or_acos01(a);
}

/* Longest valid segments of R^3 and SO(3): out[0], out[1]. */
OR_EXPORT void or_ompl_lvs(const double lo[3], const double hi[3], double cdres, double out[2])
{
	double e = 0.0;
	for (int c = 0; c < 3; c++) {
		const double d = hi[c] - lo[c];
		e = e + d * d;
	}
	out[0] = sqrt(e) * cdres;
	out[1] = OR_PIO2_HI * cdres;
}

/* The compound space's validSegmentCount(a, b). */
OR_EXPORT int64_t or_ompl_segment_count(const double a[7], const double b[7], const double lvs[2])
{
	const double dx = a[0] - b[0], dy = a[1] - b[1], dz = a[2] - b[2];
	const double dr = sqrt((dx * dx + dy * dy) + dz * dz);
	const double ds = or_ompl_arc(or_ompl_dot(a, b));
	const double nr = ceil(dr / lvs[0]), ns = ceil(ds / lvs[1]);
	return (int64_t)(nr > ns ? nr : ns);
}

/* SE3StateSpace::interpolate: R^3 linear, SO(3) slerp with `from` kept below DBL_EPSILON. */
OR_EXPORT void or_ompl_interpolate(const double a[7], const double b[7], double t, double out[7])
{
	for (int c = 0; c < 3; c++)
		out[c] = a[c] + (b[c] - a[c]) * t;
	const double dq = or_ompl_dot(a, b);
	const double theta = or_ompl_arc(dq);
	if (theta > 2.220446049250313080847e-16) {
		const double d = 1.0 / or_sin(theta);
		const double s0 = or_sin((1.0 - t) * theta);
		double s1 = or_sin(t * theta);
		if (dq < 0.0)
			s1 = -s1;
		for (int c = 3; c < 7; c++)
			out[c] = (a[c] * s0 + b[c] * s1) * d;
	} else {
		for (int c = 3; c < 7; c++)
			out[c] = a[c];
	}
}

/* The states checkMotion(a, b) checks, b first, then k = 1 .. nd - 1; returns their
 * number and writes at most cap of them. */
OR_EXPORT int64_t or_ompl_motion_states(const double a[7], const double b[7], const double lvs[2], int64_t cap,
                                        double *out)
{
	const int64_t nd = or_ompl_segment_count(a, b, lvs);
	const int64_t m = nd >= 2 ? nd : 1;
	for (int c = 0; c < 7 && cap > 0; c++)
		out[c] = b[c];
	for (int64_t k = 1; k < m && k < cap; k++)
		or_ompl_interpolate(a, b, (double)k / (double)nd, out + 7 * k);
	return m;
}

/* Hamilton product a * b, quaternions (w, x, y, z). */
static void or_quat_mul(const double a[4], const double b[4], double o[4])
{
	o[0] = ((a[0] * b[0] - a[1] * b[1]) - a[2] * b[2]) - a[3] * b[3];
	o[1] = ((a[0] * b[1] + a[1] * b[0]) + a[2] * b[3]) - a[3] * b[2];
	o[2] = ((a[0] * b[2] - a[1] * b[3]) + a[2] * b[0]) + a[3] * b[1];
	o[3] = ((a[0] * b[3] + a[1] * b[2]) - a[2] * b[1]) + a[3] * b[0];
}

/* decompose / compose (osr_state.cc:85-119): the rotation normalised each way. */
static void or_decompose(const double q[7], double t[3], double rot[4])
{
	t[0] = q[0]; t[1] = q[1]; t[2] = q[2];
	const double r[4] = { q[3], q[4], q[5], q[6] };
	or_quat_normalize(r, rot);
}

static void or_compose(const double t[3], const double rot[4], double q[7])
{
	double r[4];
	or_quat_normalize(rot, r);
	q[0] = t[0]; q[1] = t[1]; q[2] = t[2];
	q[3] = r[0]; q[4] = r[1]; q[5] = r[2]; q[6] = r[3];
}

static void or_mat_vec(const double R[9], const double v[3], double o[3])
{
	for (int i = 0; i < 3; i++)
		o[i] = (R[3 * i] * v[0] + R[3 * i + 1] * v[1]) + R[3 * i + 2] * v[2];
}

/* translateOMPLStateToUnitState (unit_world.cc:689-711) of one OMPL state (x, y, z, qx,
 * qy, qz, qw): w-first, translation scaled, applyPertubation (:713-724), then
 * t' = t - R(q) (OMPL centre - centre) scale. */
OR_EXPORT void or_ompl_to_unit(const or_world *w, const double p[7], double u[7])
{
	const double s = (double)w->scale;
	const double tmp[7] = { s * p[0], s * p[1], s * p[2], p[6], p[3], p[4], p[5] };
	double t[3], rot[4], pt[3], prot[4], qret[4], R[9], Rt[3], tret[3], a[7];
	or_decompose(tmp, t, rot);
	or_decompose(w->pert, pt, prot);
	or_quat_mul(prot, rot, qret);
	or_quat_to_matrix(prot, R);
	or_mat_vec(R, t, Rt);
	for (int c = 0; c < 3; c++) tret[c] = pt[c] + Rt[c];
	or_compose(tret, qret, a);
	double dc[3], Rd[3], t2[3];
	for (int c = 0; c < 3; c++) dc[c] = (double)(w->ompl_center[c] - w->center[c]) * s;
	or_decompose(a, t, rot);
	or_quat_to_matrix(rot, R);
	or_mat_vec(R, dc, Rd);
	for (int c = 0; c < 3; c++) t2[c] = t[c] - Rd[c];
	or_compose(t2, rot, u);
}

static int or_finite7(const double *q)
{
	for (int c = 0; c < 7; c++)
		if (!isfinite(q[c]))
			return 0;
	return 1;
}

/* OmplDriver::validateMotionPairs (ompldriver.cc:597-621) for n OMPL-frame motions, as
 * OMPL's DiscreteMotionValidator::checkMotion runs it: the target state first, then the
 * middle state of each index range in a FIFO that starts with [1, nd - 1] and splits each
 * checked range in two, stopping at the first colliding state.  valid[i] = 1 when none
 * collides; checks[i] = the states checked.  A motion with a non-finite component gets 0
 * and no checks. */
OR_EXPORT void or_ompl_check_motions(const or_world *w, const double *from, const double *to, int64_t n,
                                     const double lvs[2], uint8_t *valid, int64_t *checks, int nthreads)
{
#ifdef _OPENMP
	if (nthreads > 0) omp_set_num_threads(nthreads);
#pragma omp parallel for schedule(dynamic, 16)
#endif
	for (int64_t i = 0; i < n; i++) {
		const double *a = from + 7 * i, *b = to + 7 * i;
		valid[i] = 0;
		checks[i] = 0;
		if (!or_finite7(a) || !or_finite7(b))
			continue;
		double u[7], s[7];
		or_ompl_to_unit(w, b, u);
		checks[i] = 1;
		if (!or_is_valid(w, u, 0))
			continue;
		const int64_t nd = or_ompl_segment_count(a, b, lvs);
		int ok = 1;
		if (nd >= 2) {
			int64_t *q = (int64_t *)malloc(sizeof(int64_t) * 2 * (size_t)nd);
			int64_t head = 0, tail = 0;
			q[0] = 1; q[1] = nd - 1;
			tail = 1;
			while (head < tail) {
				const int64_t f = q[2 * (head % nd)], l = q[2 * (head % nd) + 1];
				const int64_t mid = (f + l) / 2;
				or_ompl_interpolate(a, b, (double)mid / (double)nd, s);
				or_ompl_to_unit(w, s, u);
				checks[i]++;
				if (!or_is_valid(w, u, 0)) {
					ok = 0;
					break;
				}
				head++;
				if (f < mid) {
					q[2 * (tail % nd)] = f; q[2 * (tail % nd) + 1] = mid - 1;
					tail++;
				}
				if (l > mid) {
					q[2 * (tail % nd)] = mid + 1; q[2 * (tail % nd) + 1] = l;
					tail++;
				}
			}
			free(q);
		}
		valid[i] = (uint8_t)ok;
	}
}

/* ------------------------------------------------------------------------ */
/* Key-configuration states (unit_world.cc:1294-1389)                        */
/* ------------------------------------------------------------------------ */

/* The candidate state of UnitWorld::enumFreeConfiguration /
 * sampleFreeConfiguration for one surface pair and one spin, in Eigen's
 * published forms (unit_world.cc:1301-1330 calls them): the robot point plus
 * margin x normal goes to the environment point plus margin x normal, after
 * rot_1 = Quaternion::setFromTwoVectors(rob normal, -env normal) (normalise
 * both, c = v0.v1; w = s / 2 and vec = (v0 x v1) * (1 / s) with
 * s = sqrt((1 + c) * 2); for c < -1 + 1e-12 a half turn about an axis
 * perpendicular to v0) and rot_2 = AngleAxis(angle, env normal)
 * = (cos(angle / 2), sin(angle / 2) * normal), rot_accum = rot_2 * rot_1;
 * trans = env_o - rot_accum * rob_o with Eigen's quaternion-vector product
 * (uv = u x v, uv += uv, v + w uv + u x uv); compose normalises the rotation.
 * hc, hs: the half angle's cosine and sine. */
static double or_norm3(const double v[3]) { return sqrt((v[0] * v[0] + v[1] * v[1]) + v[2] * v[2]); }

static void or_keyconf_state(const double rp[3], const double rn[3], const double ep[3], const double en[3],
                             double margin, double hc, double hs, double out[7])
{
	double rob_o[3], env_o[3], v0[3], v1[3], r1[4];
	for (int i = 0; i < 3; i++) {
		rob_o[i] = rp[i] + rn[i] * margin;
		env_o[i] = ep[i] + en[i] * margin;
	}
	const double na = or_norm3(rn);
	const double neg[3] = { -en[0], -en[1], -en[2] };
	const double nb = or_norm3(neg);
	for (int i = 0; i < 3; i++) {
		v0[i] = rn[i] / na;
		v1[i] = neg[i] / nb;
	}
	const double c = (v0[0] * v1[0] + v0[1] * v1[1]) + v0[2] * v1[2];
	if (c < -1.0 + 1e-12) {
		int k = 0;
		if (fabs(v0[1]) < fabs(v0[k])) k = 1;
		if (fabs(v0[2]) < fabs(v0[k])) k = 2;
		const double e[3] = { k == 0 ? 1.0 : 0.0, k == 1 ? 1.0 : 0.0, k == 2 ? 1.0 : 0.0 };
		double ax[3];
		or_cross3(v0, e, ax);
		const double n = or_norm3(ax);
		r1[0] = 0.0; r1[1] = ax[0] / n; r1[2] = ax[1] / n; r1[3] = ax[2] / n;
	} else {
		const double s = sqrt((1.0 + c) * 2.0);
		const double invs = 1.0 / s;
		double ax[3];
		or_cross3(v0, v1, ax);
		r1[0] = s * 0.5; r1[1] = ax[0] * invs; r1[2] = ax[1] * invs; r1[3] = ax[2] * invs;
	}
	const double r2[4] = { hc, hs * en[0], hs * en[1], hs * en[2] };
	double acc[4];
	acc[0] = ((r2[0] * r1[0] - r2[1] * r1[1]) - r2[2] * r1[2]) - r2[3] * r1[3];
	acc[1] = ((r2[0] * r1[1] + r2[1] * r1[0]) + r2[2] * r1[3]) - r2[3] * r1[2];
	acc[2] = ((r2[0] * r1[2] - r2[1] * r1[3]) + r2[2] * r1[0]) + r2[3] * r1[1];
	acc[3] = ((r2[0] * r1[3] + r2[1] * r1[2]) - r2[2] * r1[1]) + r2[3] * r1[0];
	const double u[3] = { acc[1], acc[2], acc[3] };
	double t[3], ut[3];
	or_cross3(u, rob_o, t);
	for (int i = 0; i < 3; i++)
		t[i] = t[i] + t[i];
	or_cross3(u, t, ut);
	for (int i = 0; i < 3; i++)
		out[i] = env_o[i] - ((rob_o[i] + acc[0] * t[i]) + ut[i]);
	or_quat_normalize(acc, out + 3);
}

/* The states of npairs surface pairs x nspins spins ([npairs x nspins x 7]);
 * the half-angle tables are [nspins] (per_pair 0) or [npairs x nspins]. */
OR_EXPORT void or_keyconf_states(const double *rp, const double *rn, const double *ep, const double *en, int64_t np,
                                 double margin, const double *hc, const double *hs, int64_t na, int per_pair,
                                 double *out, int nthreads)
{
	if (nthreads > 0)
		omp_set_num_threads(nthreads);
#pragma omp parallel for schedule(static)
	for (int64_t i = 0; i < np * na; i++) {
		const int64_t p = i / na, a = i % na, k = per_pair ? i : a;
		or_keyconf_state(rp + 3 * p, rn + 3 * p, ep + 3 * p, en + 3 * p, margin, hc[k], hs[k], out + 7 * i);
	}
}
