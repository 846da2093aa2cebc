// disentangled_bounds.cc -- pwf::boxes_disjoint32 (the FP32 isDisentangled test)
// against pwm::boxes_disjoint (FP64, the verdict of record) on states moved by
// bisection to just either side of the boxes' contact, and on random states.
// Host-only; built with g++.
//
// usage: disentangled_bounds <pairs> <seed> <slack>; prints
// "wrong W certified C undecided U states S far_undecided F far_states N"
// (far: the two states per pair drawn away from the contact) and exits 1 if W > 0.
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>

#include "pw_filter.cuh"

static uint64_t rng_state = 88172645463325252ull;
static uint64_t next_u64()
{
	rng_state ^= rng_state << 13;
	rng_state ^= rng_state >> 7;
	rng_state ^= rng_state << 17;
	return rng_state;
}
static double uniform() { return (double)(next_u64() >> 11) * (1.0 / 9007199254740992.0); }
static double normal()
{
	const double u1 = uniform() + 1e-300, u2 = uniform();
	return std::sqrt(-2.0 * std::log(u1)) * std::cos(6.283185307179586 * u2);
}

static void random_quat(double q[4])
{
	double n = 0;
	for (int k = 0; k < 4; k++) {
		q[k] = normal();
		n += q[k] * q[k];
	}
	n = std::sqrt(n);
	for (int k = 0; k < 4; k++)
		q[k] /= n;
}

static void quat_matrix(const double q[4], double R[9])
{
	const double w = q[0], x = q[1], y = q[2], z = q[3];
	R[0] = 1 - 2 * (y * y + z * z); R[1] = 2 * (x * y - w * z); R[2] = 2 * (x * z + w * y);
	R[3] = 2 * (x * y + w * z); R[4] = 1 - 2 * (x * x + z * z); R[5] = 2 * (y * z - w * x);
	R[6] = 2 * (x * z - w * y); R[7] = 2 * (y * z + w * x); R[8] = 1 - 2 * (x * x + y * y);
}

struct Boxes {
	double rc[3], rh[3], Re[9], te[3], ec[3], eh[3];
	pwf::DisBoxes32 b32;
};

static void make_boxes(Boxes &B)
{
	const double s = std::exp(normal());                  // scene scale around 1
	for (int c = 0; c < 3; c++) {
		B.rc[c] = 0.3 * s * normal();
		B.rh[c] = s * (0.01 + uniform());
		B.ec[c] = 0.3 * s * normal();
		B.eh[c] = s * (0.01 + uniform());
		B.te[c] = (next_u64() & 1) ? 0.0 : 0.2 * s * normal();
	}
	double qe[4] = { 1, 0, 0, 0 };
	if (next_u64() & 1)
		random_quat(qe);
	quat_matrix(qe, B.Re);
	double ce[3];
	pwm::xform_point(B.Re, B.te, B.ec, ce);
	float cabs = 0.f;
	for (int c = 0; c < 3; c++) {
		B.b32.rc[c] = (float)B.rc[c];
		B.b32.rh[c] = (float)B.rh[c];
		B.b32.eh[c] = (float)B.eh[c];
		B.b32.ce[c] = (float)ce[c];
		cabs = std::fmax(cabs, std::fabs(B.b32.ce[c]));
	}
	for (int i = 0; i < 9; i++)
		B.b32.Re[i] = (float)B.Re[i];
	B.b32.ce_abs = cabs * (1.f + 1e-6f);
}

int main(int argc, char **argv)
{
	const long pairs = argc > 1 ? atol(argv[1]) : 10000;
	rng_state ^= (uint64_t)(argc > 2 ? atol(argv[2]) : 1) * 0x9E3779B97F4A7C15ull;
	const float slack = argc > 3 ? (float)atof(argv[3]) : 1.f;
	long wrong = 0, certified = 0, undecided = 0, states = 0, far_und = 0, far_states = 0;
	// pwf::f32_trunc: truncation error below 2^-23 |x| in the normal FP32 range, a
	// magnitude below 2^-126 under it, a finite magnitude of at least 2^127 above it
	auto conv_ok = [](double x) {
		const float f = pwf::f32_trunc(x);
		const double ax = std::fabs(x), af = std::fabs((double)f);
		if (!std::isfinite(f))
			return false;
		if (!(ax < 1e300) || ax >= std::ldexp(1.0, 128))   // non-finite or beyond FP32
			return af >= std::ldexp(1.0, 127);
		if (ax < std::ldexp(1.0, -126))
			return af < std::ldexp(1.0, -126);
		return af <= ax && ax - af < std::ldexp(ax, -23) && (x == 0.0 || std::signbit(x) == std::signbit(f));
	};
	const double specials[] = { 0.0, -0.0, 1.0, -1.0, std::ldexp(1.0, -126), std::ldexp(1.0, -127),
		                        std::ldexp(1.0, -149), 1e-300, std::ldexp(1.0, 127), std::ldexp(1.0, 128),
		                        -std::ldexp(1.0, 128), 1e300, HUGE_VAL, -HUGE_VAL, NAN,
		                        std::nextafter(std::ldexp(1.0, 128), 0.0), std::nextafter(1.0, 2.0) };
	for (double x : specials)
		if (!conv_ok(x))
			wrong++;
	for (long i = 0; i < 200000; i++) {
		const double x = std::ldexp(uniform() + 0.5, (int)(next_u64() % 600) - 300) * ((next_u64() & 1) ? 1 : -1);
		if (!conv_ok(x))
			wrong++;
	}
	double prev[7] = { 0, 0, 0, 1, 0, 0, 0 };
	auto check = [&](const Boxes &B, const double q[7]) {
		const int ref = pwm::boxes_disjoint(q, B.rc, B.rh, B.Re, B.te, B.ec, B.eh);
		// the two-state form on (the previous state, this one) gives the one-state verdicts
		int va, vb;
		pwf::boxes_disjoint32x2<true>(prev, q, B.b32, va, vb, slack);
		if (va != pwf::boxes_disjoint32<true>(prev, B.b32, slack) || vb != pwf::boxes_disjoint32<true>(q, B.b32, slack))
			wrong++;
		for (int c = 0; c < 7; c++)
			prev[c] = q[c];
		// the general form, and the identity-rotation form where Re is exactly the identity
		const bool ident = B.Re[0] == 1.0 && B.Re[4] == 1.0 && B.Re[8] == 1.0 && B.Re[1] == 0.0 && B.Re[2] == 0.0 &&
		                   B.Re[3] == 0.0 && B.Re[5] == 0.0 && B.Re[6] == 0.0 && B.Re[7] == 0.0;
		const int v = pwf::boxes_disjoint32<true>(q, B.b32, slack);
		if (ident && pwf::boxes_disjoint32<false>(q, B.b32, slack) != v)
			wrong++;
		states++;
		if (v < 0) {
			undecided++;
			return;
		}
		certified++;
		if (v != ref)
			wrong++;
	};
	for (long p = 0; p < pairs; p++) {
		Boxes B;
		make_boxes(B);
		double q[7];
		double rq[4];
		random_quat(rq);
		// a quaternion that is not normalised, as states may come
		const double sc = 0.5 + uniform();
		for (int k = 0; k < 4; k++)
			q[3 + k] = rq[k] * sc;
		// direction of travel of the robot box's centre, from overlap (near the env centre) outwards
		double v[3], base[3], ce[3];
		pwm::xform_point(B.Re, B.te, B.ec, ce);
		for (int c = 0; c < 3; c++) {
			v[c] = normal();
			base[c] = ce[c];
		}
		// t puts the placed robot centre at base + s v: t = base + s v - R rc
		double R[9], tt[3], Rrc[3];
		pwm::state_transform(q, R, tt);
		const double zero[3] = { 0, 0, 0 };
		pwm::xform_point(R, zero, B.rc, Rrc);
		auto at = [&](double s, double out[7]) {
			for (int c = 0; c < 3; c++)
				out[c] = base[c] + s * v[c] - Rrc[c];
			for (int k = 3; k < 7; k++)
				out[k] = q[k];
		};
		double lo = 0.0, hi = 1.0, st[7];
		at(lo, st);
		if (pwm::boxes_disjoint(st, B.rc, B.rh, B.Re, B.te, B.ec, B.eh))
			continue;                                   // centres together yet disjoint: degenerate draw
		for (int g = 0; g < 60; g++) {
			at(hi, st);
			if (pwm::boxes_disjoint(st, B.rc, B.rh, B.Re, B.te, B.ec, B.eh))
				break;
			hi *= 2.0;
		}
		for (int it = 0; it < 80 && hi - lo > 1e-17 * hi; it++) {
			const double mid = 0.5 * (lo + hi);
			at(mid, st);
			if (pwm::boxes_disjoint(st, B.rc, B.rh, B.Re, B.te, B.ec, B.eh))
				hi = mid;
			else
				lo = mid;
		}
		// both sides of the contact, points near it at several distances, and far states
		const double offs[] = { 0.0, 1e-12, 1e-9, 1e-7, 1e-6, 1e-5, 1e-4, 1e-3, 1e-2, 1e-1 };
		for (double o : offs) {
			at(lo * (1.0 - o), st);
			check(B, st);
			at(hi * (1.0 + o), st);
			check(B, st);
		}
		const long u0 = undecided;
		at(hi * (1.0 + 10.0 * uniform()), st);
		check(B, st);
		at(lo * uniform(), st);
		check(B, st);
		far_und += undecided - u0;
		far_states += 2;
	}
	printf("wrong %ld certified %ld undecided %ld states %ld far_undecided %ld far_states %ld\n", wrong, certified,
	       undecided, states, far_und, far_states);
	return wrong ? 1 : 0;
}
