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

int main(int argc, char **argv)
{
	const long n = argc > 1 ? atol(argv[1]) : 2000000;
	const unsigned seed = argc > 2 ? (unsigned)atoi(argv[2]) : 1u;
	std::mt19937_64 rng(seed);
	std::uniform_real_distribution<double> U(-1.0, 1.0), P(0.0, 1.0);
	long uncertain = 0, fviol = 0, bviol = 0, hits = 0, certified_hits = 0, gviol = 0, sviol = 0, gaps = 0;
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
		const float sep = sat_sep32(A0, A1, B0, B1, Q.q[0], Q.q[1], Q.q[2], Q.q[3]);
		if (truth && sep > 0.f) {
			bviol++;
			if (bviol < 5) printf("box violation: case %ld L=%g off=%g\n", it, L, off);
		}
		if (!truth && sep > 0.f && (double)sep > tri_dist(V, Uw) * (1 + 1e-9) + 1e-14) {
			sviol++;
			if (sviol < 5) printf("box separation above the distance: case %ld sep=%g\n", it, sep);
		}
	}
	printf("gaps %ld gap_violations %ld separation_violations %ld\n", gaps, gviol, sviol);
	printf("cases %ld hits %ld certified_hits %ld uncertain %ld filter_violations %ld box_violations %ld\n", n, hits,
	       certified_hits, uncertain, fviol, bviol + gviol + sviol);
	return (fviol || bviol || gviol || sviol) ? 1 : 0;
}
