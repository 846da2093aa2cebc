// Host harness: the FP32 box and triangle tests against the FP64 triangle test.
//
// For random triangle pairs placed near contact (offsets from 1e-12 to 1 of
// the triangle size, several scales, random and slightly non-unit rotations),
// every verdict the FP32 filter certifies must equal the FP64 verdict, and the
// box test must never separate boxes of triangles that FP64 finds touching.
// Prints: cases, uncertain, filter violations, box violations.
#include <cstdio>
#include <cstdlib>
#include <cmath>
#include <random>

#include "pw_filter.cuh"

using namespace pwf;

static float rd(double x) { float f = (float)x; if ((double)f > x) f = nextafterf(f, -INFINITY); return f; }
static float ru(double x) { float f = (float)x; if ((double)f < x) f = nextafterf(f, INFINITY); return f; }


// Exact distances in FP64 (closest points, Ericson, Real-Time Collision Detection 5.1).
static void sub(const double *a, const double *b, double *o) { for (int i = 0; i < 3; i++) o[i] = a[i] - b[i]; }
static double dot(const double *a, const double *b) { return a[0] * b[0] + a[1] * b[1] + a[2] * b[2]; }
static double clamp01(double x) { return x < 0 ? 0 : (x > 1 ? 1 : x); }

static double point_tri(const double *p, const double *a, const double *b, const double *c)
{
	double ab[3], ac[3], ap[3], q[3];
	sub(b, a, ab); sub(c, a, ac); sub(p, a, ap);
	const double d1 = dot(ab, ap), d2 = dot(ac, ap);
	if (d1 <= 0 && d2 <= 0) { sub(p, a, q); return sqrt(dot(q, q)); }
	double bp[3]; sub(p, b, bp);
	const double d3 = dot(ab, bp), d4 = dot(ac, bp);
	if (d3 >= 0 && d4 <= d3) { sub(p, b, q); return sqrt(dot(q, q)); }
	const double vc = d1 * d4 - d3 * d2;
	if (vc <= 0 && d1 >= 0 && d3 <= 0) {
		const double v = d1 / (d1 - d3);
		for (int i = 0; i < 3; i++) q[i] = p[i] - (a[i] + v * ab[i]);
		return sqrt(dot(q, q));
	}
	double cp[3]; sub(p, c, cp);
	const double d5 = dot(ab, cp), d6 = dot(ac, cp);
	if (d6 >= 0 && d5 <= d6) { sub(p, c, q); return sqrt(dot(q, q)); }
	const double vb = d5 * d2 - d1 * d6;
	if (vb <= 0 && d2 >= 0 && d6 <= 0) {
		const double w = d2 / (d2 - d6);
		for (int i = 0; i < 3; i++) q[i] = p[i] - (a[i] + w * ac[i]);
		return sqrt(dot(q, q));
	}
	const double va = d3 * d6 - d5 * d4;
	if (va <= 0 && (d4 - d3) >= 0 && (d5 - d6) >= 0) {
		const double w = (d4 - d3) / ((d4 - d3) + (d5 - d6));
		for (int i = 0; i < 3; i++) q[i] = p[i] - (b[i] + w * (c[i] - b[i]));
		return sqrt(dot(q, q));
	}
	const double den = 1.0 / (va + vb + vc);
	const double v = vb * den, w = vc * den;
	for (int i = 0; i < 3; i++) q[i] = p[i] - (a[i] + ab[i] * v + ac[i] * w);
	return sqrt(dot(q, q));
}

static double seg_seg(const double *p1, const double *q1, const double *p2, const double *q2)
{
	double d1[3], d2[3], r[3];
	sub(q1, p1, d1); sub(q2, p2, d2); sub(p1, p2, r);
	const double a = dot(d1, d1), e = dot(d2, d2), f = dot(d2, r);
	double s, t;
	const double c = dot(d1, r), b = dot(d1, d2), den = a * e - b * b;
	s = den != 0 ? clamp01((b * f - c * e) / den) : 0;
	t = (b * s + f) / e;
	if (t < 0) { t = 0; s = clamp01(-c / a); }
	else if (t > 1) { t = 1; s = clamp01((b - c) / a); }
	double x[3];
	for (int i = 0; i < 3; i++) x[i] = (p1[i] + d1[i] * s) - (p2[i] + d2[i] * t);
	return sqrt(dot(x, x));
}

static double tri_dist(double V[3][3], double U[3][3])
{
	double d = 1e300;
	for (int k = 0; k < 3; k++) {
		d = fmin(d, point_tri(V[k], U[0], U[1], U[2]));
		d = fmin(d, point_tri(U[k], V[0], V[1], V[2]));
	}
	for (int i = 0; i < 3; i++)
		for (int j = 0; j < 3; j++)
			d = fmin(d, seg_seg(V[i], V[(i + 1) % 3], U[j], U[(j + 1) % 3]));
	return d;
}

// An oriented box around np points, fitted as the BVH build fits a node: principal
// axes of the points (pwm::jacobi_eigen3), FP32 centre of the projections' range,
// half-extents about that centre measured in FP64 and rounded up with the same
// margin.  E receives the FP64 frame.
static void fit_obb(const double (*p)[3], int np, float4 &c4, float4 &h4, float4 rows[3], double E[9])
{
	double mu[3] = { 0, 0, 0 };
	for (int k = 0; k < np; k++)
		for (int a = 0; a < 3; a++) mu[a] += p[k][a] / np;
	double S[6] = { 0, 0, 0, 0, 0, 0 };
	for (int k = 0; k < np; k++) {
		const double d[3] = { p[k][0] - mu[0], p[k][1] - mu[1], p[k][2] - mu[2] };
		S[0] += d[0] * d[0] / np; S[1] += d[1] * d[1] / np; S[2] += d[2] * d[2] / np;
		S[3] += d[0] * d[1] / np; S[4] += d[0] * d[2] / np; S[5] += d[1] * d[2] / np;
	}
	pwm::jacobi_eigen3(S, E);
	double pmin[3] = { 1e300, 1e300, 1e300 }, pmax[3] = { -1e300, -1e300, -1e300 };
	for (int k = 0; k < np; k++)
		for (int a = 0; a < 3; a++) {
			const double pr = E[3 * a] * p[k][0] + E[3 * a + 1] * p[k][1] + E[3 * a + 2] * p[k][2];
			pmin[a] = std::fmin(pmin[a], pr);
			pmax[a] = std::fmax(pmax[a], pr);
		}
	float c[3];
	for (int k = 0; k < 3; k++) {
		double ck = 0;
		for (int a = 0; a < 3; a++) ck += E[3 * a + k] * 0.5 * (pmin[a] + pmax[a]);
		c[k] = (float)ck;
	}
	double h[3] = { 0, 0, 0 }, dmax = 0;
	for (int k = 0; k < np; k++) {
		const double d0 = p[k][0] - c[0], d1 = p[k][1] - c[1], d2 = p[k][2] - c[2];
		dmax = std::fmax(dmax, std::fabs(d0) + std::fabs(d1) + std::fabs(d2));
		for (int a = 0; a < 3; a++)
			h[a] = std::fmax(h[a], std::fabs(E[3 * a] * d0 + E[3 * a + 1] * d1 + E[3 * a + 2] * d2));
	}
	const double cinf = std::fmax(std::fmax(std::fabs((double)c[0]), std::fabs((double)c[1])), std::fabs((double)c[2]));
	const double pad = 1e-14 * (dmax + 2.0 * cinf) + 1e-300;
	float hf[3];
	for (int a = 0; a < 3; a++) hf[a] = ru(h[a] * (1.0 + 1e-14) + pad);
	c4 = make_float4(c[0], c[1], c[2], 0.f);
	h4 = make_float4(hf[0], hf[1], hf[2], 0.f);
	for (int a = 0; a < 3; a++) rows[a] = make_float4((float)E[3 * a], (float)E[3 * a + 1], (float)E[3 * a + 2], 0.f);
}

// Smallest overlap, over the 15 separating axes, of two exact oriented boxes in
// FP64 (axes as rows): negative when some axis separates them.
static double obb_overlap64(const double *ca, const double *Ea, const double *ha, const double *cb, const double *Eb,
                            const double *hb)
{
	double R[3][3], AR[3][3], T[3];
	const double d[3] = { cb[0] - ca[0], cb[1] - ca[1], cb[2] - ca[2] };
	for (int i = 0; i < 3; i++) {
		T[i] = Ea[3 * i] * d[0] + Ea[3 * i + 1] * d[1] + Ea[3 * i + 2] * d[2];
		for (int j = 0; j < 3; j++) {
			R[i][j] = Ea[3 * i] * Eb[3 * j] + Ea[3 * i + 1] * Eb[3 * j + 1] + Ea[3 * i + 2] * Eb[3 * j + 2];
			AR[i][j] = std::fabs(R[i][j]);
		}
	}
	double m = 1e300;
	for (int i = 0; i < 3; i++)
		m = std::fmin(m, ha[i] + hb[0] * AR[i][0] + hb[1] * AR[i][1] + hb[2] * AR[i][2] - std::fabs(T[i]));
	for (int j = 0; j < 3; j++)
		m = std::fmin(m, hb[j] + ha[0] * AR[0][j] + ha[1] * AR[1][j] + ha[2] * AR[2][j] -
		                     std::fabs(T[0] * R[0][j] + T[1] * R[1][j] + T[2] * R[2][j]));
	for (int i = 0; i < 3; i++) {
		const int i1 = (i + 1) % 3, i2 = (i + 2) % 3;
		for (int j = 0; j < 3; j++) {
			const int j1 = (j + 1) % 3, j2 = (j + 2) % 3;
			const double len = std::sqrt(std::fmax(1e-300, 1.0 - R[i][j] * R[i][j]));
			const double t = std::fabs(T[i2] * R[i1][j] - T[i1] * R[i2][j]);
			const double ra = ha[i1] * AR[i2][j] + ha[i2] * AR[i1][j];
			const double rb = hb[j1] * AR[i][j2] + hb[j2] * AR[i][j1];
			if (len > 1e-6)
				m = std::fmin(m, (ra + rb - t) / len);
		}
	}
	return m;
}

int main(int argc, char **argv)
{
	const long n = argc > 1 ? atol(argv[1]) : 2000000;
	const unsigned seed = argc > 2 ? (unsigned)atoi(argv[2]) : 1u;
	std::mt19937_64 rng(seed);
	std::uniform_real_distribution<double> U(-1.0, 1.0), P(0.0, 1.0);
	long uncertain = 0, fviol = 0, bviol = 0, hits = 0, certified_hits = 0, gviol = 0, sviol = 0, gaps = 0;
	long oviol = 0, oseps = 0, othick = 0, otouch = 0;
	for (long it = 0; it < n; it++) {
		const double L = std::pow(10.0, -3.0 + 2.5 * P(rng));          // triangle size 1e-3 .. 0.3
		double V[3][3], x[3][3];
		const double cV[3] = { 2 * U(rng), 2 * U(rng), 2 * U(rng) };
		const double cx[3] = { 0.6 * U(rng), 0.6 * U(rng), 0.6 * U(rng) };
		for (int k = 0; k < 3; k++)
			for (int c = 0; c < 3; c++) {
				V[k][c] = cV[c] + L * U(rng);
				x[k][c] = cx[c] + L * U(rng);
			}
		// rotation: Shoemake, sometimes scaled slightly off unit length
		const double u1 = P(rng), u2 = P(rng), u3 = P(rng);
		double q[7];
		q[3] = std::sqrt(1 - u1) * std::sin(2 * M_PI * u2);
		q[4] = std::sqrt(1 - u1) * std::cos(2 * M_PI * u2);
		q[5] = std::sqrt(u1) * std::sin(2 * M_PI * u3);
		q[6] = std::sqrt(u1) * std::cos(2 * M_PI * u3);
		if (it % 7 == 0)
			for (int i = 3; i < 7; i++) q[i] *= 1.0 + 1e-7 * U(rng);
		double R[9], t0[3] = { 0, 0, 0 };
		{
			const double qq[7] = { 0, 0, 0, q[3], q[4], q[5], q[6] };
			pwm::state_transform(qq, R, t0);
		}
		// translation: a robot vertex (or the centroid) onto an env point, plus an offset
		const int kv = (int)(P(rng) * 4);
		double src[3], dst[3];
		const double a = P(rng), b = P(rng) * (1 - a);
		for (int c = 0; c < 3; c++) {
			dst[c] = V[0][c] + a * (V[1][c] - V[0][c]) + b * (V[2][c] - V[0][c]);
			src[c] = kv < 3 ? x[kv][c] : (x[0][c] + x[1][c] + x[2][c]) / 3;
		}
		double Rs[3];
		pwm::xform_point(R, t0, src, Rs);
		const double off = L * (it % 5 == 0 ? 3.0 * P(rng) : std::pow(10.0, -12.0 * P(rng)));
		for (int c = 0; c < 3; c++)
			q[c] = dst[c] - Rs[c] + off * U(rng);
		// FP64 truth with the oracle's arithmetic
		double RR[9], tt[3], Uw[3][3];
		pwm::state_transform(q, RR, tt);
		for (int k = 0; k < 3; k++)
			pwm::xform_point(RR, tt, x[k], Uw[k]);
		const int truth = pwm::tri_tri(V[0], V[1], V[2], Uw[0], Uw[1], Uw[2], 0.0);
		hits += truth;
		// FP32 data as the engine stores it
		double emax = 0, r1 = 0;
		for (int k = 0; k < 3; k++) {
			double l1 = 0;
			for (int c = 0; c < 3; c++) {
				emax = std::fmax(emax, std::fabs(V[k][c]));
				l1 += std::fabs(x[k][c]);
			}
			r1 = std::fmax(r1, l1);
		}
		QFs Q;
		make_qf(q, (float)r1 * 1.0001f, (float)emax * 1.0001f, 5.9604645e-08f * (float)emax * 1.0001f, Q);
		const float3 V0 = make_float3((float)V[0][0], (float)V[0][1], (float)V[0][2]);
		const float3 e1 = make_float3((float)(V[1][0] - V[0][0]), (float)(V[1][1] - V[0][1]), (float)(V[1][2] - V[0][2]));
		const float3 e2 = make_float3((float)(V[2][0] - V[0][0]), (float)(V[2][1] - V[0][1]), (float)(V[2][2] - V[0][2]));
		const float3 x0 = make_float3((float)x[0][0], (float)x[0][1], (float)x[0][2]);
		const float3 g1 = make_float3((float)(x[1][0] - x[0][0]), (float)(x[1][1] - x[0][1]), (float)(x[1][2] - x[0][2]));
		const float3 g2 = make_float3((float)(x[2][0] - x[0][0]), (float)(x[2][1] - x[0][1]), (float)(x[2][2] - x[0][2]));
		float gap = 0.f;
		const int r = tri_filter(V0, e1, e2, x0, g1, g2, Q.q[0], Q.q[1], Q.q[2], Q.q[3], Q.q[4].x, &gap);
		if (r == 2) uncertain++;
		if (r == 1) certified_hits++;
		if (r == 0 && !truth && gap > 0.f) {
			gaps++;
			const double td = tri_dist(V, Uw);
			if ((double)gap > td * (1 + 1e-9) + 1e-14) {
				gviol++;
				if (gviol < 5) printf("gap violation: case %ld gap=%g dist=%g\n", it, gap, td);
			}
		}
		if ((r == 0 && truth) || (r == 1 && !truth)) {
			fviol++;
			if (fviol < 5) printf("filter violation: case %ld r=%d truth=%d L=%g off=%g\n", it, r, truth, L, off);
		}
		// conservative boxes (directed rounding) of the two triangles, centre/half-extent form
		float4 A0, A1, B0, B1;
		{
			float c[3], h[3];
			for (int cc = 0; cc < 3; cc++) {
				double lo = std::fmin(std::fmin(V[0][cc], V[1][cc]), V[2][cc]);
				double hi = std::fmax(std::fmax(V[0][cc], V[1][cc]), V[2][cc]);
				const float l = rd(lo), hh = ru(hi);
				c[cc] = (float)(0.5 * ((double)l + (double)hh));
				h[cc] = ru(std::fmax((double)hh - c[cc], c[cc] - (double)l));
			}
			A0 = make_float4(c[0], c[1], c[2], 0.f);
			A1 = make_float4(h[0], h[1], h[2], 0.f);
			for (int cc = 0; cc < 3; cc++) {
				double lo = std::fmin(std::fmin(x[0][cc], x[1][cc]), x[2][cc]);
				double hi = std::fmax(std::fmax(x[0][cc], x[1][cc]), x[2][cc]);
				const float l = rd(lo), hh = ru(hi);
				c[cc] = (float)(0.5 * ((double)l + (double)hh));
				h[cc] = ru(std::fmax((double)hh - c[cc], c[cc] - (double)l));
			}
			B0 = make_float4(c[0], c[1], c[2], 0.f);
			B1 = make_float4(h[0], h[1], h[2], 0.f);
		}
		const float sep = sat_sep32<true>(A0, A1, B0, B1, Q.q[0], Q.q[1], Q.q[2], Q.q[3]);
		// the branch-free form: the same sign, and its bound (the largest axis's) is a bound too
		const float sepbf = sat_sep32<false>(A0, A1, B0, B1, Q.q[0], Q.q[1], Q.q[2], Q.q[3]);
		if ((sepbf > 0.f) != (sep > 0.f) ||
		    (!truth && sepbf > 0.f && (double)sepbf > tri_dist(V, Uw) * (1 + 1e-9) + 1e-14))
			sviol++;
		{
			// a larger rotation error bound only widens the slack, up to one too large for the
			// scaled axes (shrink <= 0): both forms agree, and neither separates touching boxes
			float4 Q3 = Q.q[3];
			Q3.x = Q3.x + 0.75f * (float)P(rng);
			const float s1 = sat_sep32<true>(A0, A1, B0, B1, Q.q[0], Q.q[1], Q.q[2], Q3);
			const float s2 = sat_sep32<false>(A0, A1, B0, B1, Q.q[0], Q.q[1], Q.q[2], Q3);
			if ((s1 > 0.f) != (s2 > 0.f) || (truth && (s1 > 0.f || s2 > 0.f)))
				sviol++;
		}
		if (truth && sep > 0.f) {
			bviol++;
			if (bviol < 5) printf("box violation: case %ld L=%g off=%g\n", it, L, off);
		}
		if (!truth && sep > 0.f && (double)sep > tri_dist(V, Uw) * (1 + 1e-9) + 1e-14) {
			sviol++;
			if (sviol < 5) printf("box separation above the distance: case %ld sep=%g\n", it, sep);
		}
		// oriented boxes of the two triangles: a certified separation needs separate triangles
		{
			float4 oA0, oA1, oB0, oB1, oE[3], oG[3];
			double EE[9], EG[9];
			fit_obb(V, 3, oA0, oA1, oE, EE);
			fit_obb(x, 3, oB0, oB1, oG, EG);
			const float osep = sat_sep32_obb<true>(oA0, oA1, oE[0], oE[1], oE[2], oB0, oB1, oG[0], oG[1], oG[2], Q.q[0],
			                                 Q.q[1], Q.q[2], Q.q[3]);
			const float osepbf = sat_sep32_obb<false>(oA0, oA1, oE[0], oE[1], oE[2], oB0, oB1, oG[0], oG[1], oG[2],
			                                          Q.q[0], Q.q[1], Q.q[2], Q.q[3]);
			if ((osepbf > 0.f) != (osep > 0.f) ||
			    (!truth && osepbf > 0.f && (double)osepbf > tri_dist(V, Uw) * (1 + 1e-9) + 1e-14))
				oviol++;
			float4 Q3 = Q.q[3];
			Q3.x = Q3.x + 0.5f * (float)P(rng);
			const float o1 = sat_sep32_obb<true>(oA0, oA1, oE[0], oE[1], oE[2], oB0, oB1, oG[0], oG[1], oG[2], Q.q[0], Q.q[1],
			                               Q.q[2], Q3);
			const float o2 = sat_sep32_obb<false>(oA0, oA1, oE[0], oE[1], oE[2], oB0, oB1, oG[0], oG[1], oG[2], Q.q[0],
			                                      Q.q[1], Q.q[2], Q3);
			if ((o1 > 0.f) != (o2 > 0.f) || (truth && (o1 > 0.f || o2 > 0.f)))
				oviol++;
			if (osep > 0.f) {
				oseps++;
				if (truth || (double)osep > tri_dist(V, Uw) * (1 + 1e-9) + 1e-14) {
					oviol++;
					if (oviol < 5) printf("oriented box violation: case %ld osep=%g truth=%d\n", it, osep, truth);
				}
			}
		}
		// thick oriented boxes (12 points around each triangle): a certified separation needs the
		// exact boxes (FP64 frames, the robot box placed by the FP64 transform) apart
		if (it % 4 == 0) {
			double pe[12][3], pr[12][3];
			const double sp = L * (0.2 + 2.0 * P(rng));
			for (int k = 0; k < 12; k++)
				for (int c = 0; c < 3; c++) {
					pe[k][c] = V[k % 3][c] + sp * U(rng);
					pr[k][c] = x[k % 3][c] + sp * U(rng);
				}
			float4 tA0, tA1, tB0, tB1, tE[3], tG[3];
			double EE[9], EG[9];
			fit_obb(pe, 12, tA0, tA1, tE, EE);
			fit_obb(pr, 12, tB0, tB1, tG, EG);
			const float tsep = sat_sep32_obb<true>(tA0, tA1, tE[0], tE[1], tE[2], tB0, tB1, tG[0], tG[1], tG[2], Q.q[0],
			                                 Q.q[1], Q.q[2], Q.q[3]);
			if ((sat_sep32_obb<false>(tA0, tA1, tE[0], tE[1], tE[2], tB0, tB1, tG[0], tG[1], tG[2], Q.q[0], Q.q[1],
			                          Q.q[2], Q.q[3]) > 0.f) != (tsep > 0.f))
				oviol++;
			const double ca[3] = { tA0.x, tA0.y, tA0.z }, ha[3] = { tA1.x, tA1.y, tA1.z };
			const double hb[3] = { tB1.x, tB1.y, tB1.z }, cbl[3] = { tB0.x, tB0.y, tB0.z };
			double cb[3], Eb[9];
			pwm::xform_point(RR, tt, cbl, cb);
			for (int j = 0; j < 3; j++)
				for (int i = 0; i < 3; i++)
					Eb[3 * j + i] = RR[3 * i] * EG[3 * j] + RR[3 * i + 1] * EG[3 * j + 1] + RR[3 * i + 2] * EG[3 * j + 2];
			const double ov = obb_overlap64(ca, EE, ha, cb, Eb, hb);
			othick++;
			// the FP64 reference's own rounding is far below 1e-12 of the boxes' scale
			if (tsep > 0.f && ov > 1e-12 * (1.0 + std::fabs(cb[0]) + std::fabs(cb[1]) + std::fabs(cb[2]))) {
				oviol++;
				if (oviol < 5) printf("thick oriented box violation: case %ld tsep=%g overlap=%g\n", it, tsep, ov);
			}
			// just touching: move the robot along a random direction to the exact contact
			// (bisection on the FP64 overlap), then test a hair on the overlapping side
			if (ov > 0.0) {
				double dir[3] = { U(rng), U(rng), U(rng) };
				const double dn = std::sqrt(dir[0] * dir[0] + dir[1] * dir[1] + dir[2] * dir[2]) + 1e-300;
				for (int c = 0; c < 3; c++) dir[c] /= dn;
				auto place = [&](double sft, double *q2, double *cbw, double *Ebw) {
					for (int c = 0; c < 7; c++) q2[c] = q[c];
					for (int c = 0; c < 3; c++) q2[c] += sft * dir[c];
					double R2[9], t2[3];
					pwm::state_transform(q2, R2, t2);
					pwm::xform_point(R2, t2, cbl, cbw);
					for (int j = 0; j < 3; j++)
						for (int i = 0; i < 3; i++)
							Ebw[3 * j + i] = R2[3 * i] * EG[3 * j] + R2[3 * i + 1] * EG[3 * j + 1] + R2[3 * i + 2] * EG[3 * j + 2];
				};
				double lo = 0.0, hi = 8.0 * (sp + L) + 1.0, q2[7], cbw[3], Ebw[9];
				for (int b = 0; b < 200; b++) {
					const double mid = 0.5 * (lo + hi);
					place(mid, q2, cbw, Ebw);
					if (obb_overlap64(ca, EE, ha, cbw, Ebw, hb) > 0.0) lo = mid; else hi = mid;
					if (hi - lo <= 1e-15 * hi) break;
				}
				for (int e = 0; e < 3; e++) {
					const double back = (e == 0 ? 1e-7 : (e == 1 ? 1e-9 : 1e-11)) * (1.0 + sp);
					place(lo - back, q2, cbw, Ebw);
					if (!(obb_overlap64(ca, EE, ha, cbw, Ebw, hb) > 0.0))
						continue;   // not inside after all (the overlap is not monotone along every line)
					QFs Q2;
					make_qf(q2, (float)r1 * 1.0001f, (float)emax * 1.0001f, 5.9604645e-08f * (float)emax * 1.0001f, Q2);
					const float s2 = sat_sep32_obb<true>(tA0, tA1, tE[0], tE[1], tE[2], tB0, tB1, tG[0], tG[1], tG[2],
					                               Q2.q[0], Q2.q[1], Q2.q[2], Q2.q[3]);
					const float s2bf = sat_sep32_obb<false>(tA0, tA1, tE[0], tE[1], tE[2], tB0, tB1, tG[0], tG[1],
					                                        tG[2], Q2.q[0], Q2.q[1], Q2.q[2], Q2.q[3]);
					otouch++;
					if (s2 > 0.f || s2bf > 0.f) {
						oviol++;
						if (oviol < 5) printf("touching oriented box violation: case %ld back=%g\n", it, back);
					}
				}
			}
		}
	}
	printf("oriented_separations %ld thick_cases %ld touching_cases %ld oriented_violations %ld\n", oseps, othick, otouch,
	       oviol);
	printf("gaps %ld gap_violations %ld separation_violations %ld\n", gaps, gviol, sviol);
	printf("cases %ld hits %ld certified_hits %ld uncertain %ld filter_violations %ld box_violations %ld\n", n, hits,
	       certified_hits, uncertain, fviol, bviol + gviol + sviol + oviol);
	return (fviol || bviol || gviol || sviol || oviol) ? 1 : 0;
}
