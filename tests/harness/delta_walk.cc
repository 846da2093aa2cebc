// delta_walk.cc -- pwm::walk_delta / delta_try / delta_jump (the kernels' shortcuts for
// runs of the reference's delta updates, unit_world.cc:463-470) against the
// updates taken one at a time, bit for bit.  Host-only; built with g++
// -ffp-contract=off like the library's host code.
//
// usage: delta_walk <segments> <seed>; prints "mismatches M walks W jumped J tried R ties T"
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <vector>

#include "pw_math.cuh"

static uint64_t rng_state = 88172645463325252ull;
static uint64_t next_u64()
{
	rng_state ^= rng_state << 13;
	rng_state ^= rng_state >> 7;
	rng_state ^= rng_state << 17;
	return rng_state;
}
static double uniform() { return (double)(next_u64() >> 11) * (1.0 / 9007199254740992.0); }

// whether step / ulp(delta) falls exactly halfway between two integers (no jump then)
static bool is_tie(double delta, double step)
{
	const uint64_t eb = pwm::dbits(delta) & 0x7FF0000000000000ull;
	const double q = step / pwm::bitsd(eb - (uint64_t(52) << 52));
	return q - __builtin_floor(q) == 0.5;
}

static double pick_step()
{
	switch (next_u64() % 4) {
	case 0:   // log-uniform in [1e-4, 0.05], full random mantissa
		return 1e-4 * __builtin_exp(uniform() * __builtin_log(500.0));
	case 1: { // few mantissa bits: its last set bit falls half an ulp of some binade the walk crosses (ties)
		const int k = 8 + (int)(next_u64() % 20);
		const double m = (double)(1 + 2 * (next_u64() % 2000));
		return m * __builtin_ldexp(1.0, -k - 11);
	}
	case 2:
		return 0.001;
	default:  // an odd multiple of a small power of two near 0.001
		return (double)(2 * (next_u64() % 100000) + 1) * __builtin_ldexp(1.0, -27);
	}
}

static double pick_dist(double step)
{
	switch (next_u64() % 4) {
	case 0:
		return step * (1.0 + uniform() * 3000.0);
	case 1: { // exactly a power of two, or one ulp either side of it
		const int e = (int)(next_u64() % 6) - 3;
		const double p = __builtin_ldexp(1.0, e);
		const int s = (int)(next_u64() % 3) - 1;
		return s == 0 ? p : (s < 0 ? __builtin_nextafter(p, 0.0) : __builtin_nextafter(p, 10.0));
	}
	case 2:   // an exact multiple of the step
		return step * (double)(1 + next_u64() % 3000);
	default:
		return uniform() * 4.0 + step;
	}
}

int main(int argc, char **argv)
{
	const long n = argc > 1 ? atol(argv[1]) : 10000;
	rng_state ^= (uint64_t)(argc > 2 ? atol(argv[2]) : 1) * 0x9E3779B97F4A7C15ull;
	long mism = 0, walks = 0, jumped = 0, tried = 0, ties = 0;
	std::vector<double> seq;
	for (long i = 0; i < n; i++) {
		const double step = pick_step();
		const double dist = pick_dist(step);
		if (!(step < dist) || dist / step > 200000.0)
			continue;
		// every delta the reference loop holds, one update at a time, and the one after its end
		seq.clear();
		double d = step;
		while (d <= dist) {
			seq.push_back(d);
			d = pwm::advance_delta(d, dist, step);
		}
		seq.push_back(d);
		const long L = (long)seq.size();
		for (int t = 0; t < 24; t++) {
			const long a = (long)(next_u64() % (uint64_t)L);
			const long room = L - 1 - a;
			const int j = (int)(next_u64() % (uint64_t)(room < 40 ? room + 1 : 41));
			const double got = pwm::walk_delta(seq[a], dist, step, j);
			walks++;
			if (pwm::dbits(got) != pwm::dbits(seq[a + j]))
				mism++;
			double c;
			if (pwm::delta_jump(seq[a], dist, step, j, &c) > 0)
				jumped++;
			double r;
			if (pwm::delta_try(seq[a], dist, step, j, &r)) {
				tried++;
				if (pwm::dbits(r) != pwm::dbits(seq[a + j]))
					mism++;
			}
			ties += is_tie(seq[a], step) ? 1 : 0;
		}
		// the set-up kernel's loop: checkpoints every 32 updates, chunks far from dist in one walk
		long K = 0, bad = 0;
		d = step;
		while (d <= dist) {
			if ((K & 31) == 0) {
				if (pwm::dbits(d) != pwm::dbits(seq[K]))
					bad++;
				const float room = (float)pwm::sub(dist, d) / (float)step;
				if (room > 40.f) {
					double r;
					if (pwm::delta_try(d, dist, step, 32, &r)) {
						d = r;
					} else {
						for (int i = 0; i < 32; i++)
							d = pwm::add(d, step);
					}
					K += 32;
					continue;
				}
			}
			d = pwm::advance_delta(d, dist, step);
			K++;
		}
		if (K != L - 1 || bad)
			mism++;
		// the last delta at or below dist, found with jumps (the contact-state rebuild)
		d = step;
		for (;;) {
			double c;
			const int k = pwm::delta_jump(d, dist, step, 1 << 30, &c);
			if (k > 0) {
				d = pwm::add(d, pwm::mul((double)k, c));
				continue;
			}
			const double nx = pwm::advance_delta(d, dist, step);
			if (!(nx <= dist))
				break;
			d = nx;
		}
		if (pwm::dbits(d) != pwm::dbits(seq[L - 2]))
			mism++;
	}
	// pwm::interpolate_w (the filter frames: reciprocal slerp weights, fused
	// multiply-adds) against pwm::interpolate_p (the reference's): the translation
	// equal, the rotation's components within 2^-47, its matrix entries within 2^-43
	long interp = 0;
	for (long i = 0; i < n; i++) {
		double a[7], b[7];
		for (int c = 0; c < 3; c++) {
			a[c] = 4.0 * uniform() - 2.0;
			b[c] = 4.0 * uniform() - 2.0;
		}
		double na = 0.0, nb = 0.0;
		for (int c = 3; c < 7; c++) {
			a[c] = 2.0 * uniform() - 1.0;
			na += a[c] * a[c];
		}
		switch (next_u64() % 4) {
		case 0:   // nearly the same rotation
			for (int c = 3; c < 7; c++) b[c] = a[c] + 1e-6 * (2.0 * uniform() - 1.0);
			break;
		case 1:   // nearly the opposite quaternion (the same rotation, the other sign)
			for (int c = 3; c < 7; c++) b[c] = -a[c] + 1e-4 * (2.0 * uniform() - 1.0);
			break;
		default:
			for (int c = 3; c < 7; c++) b[c] = 2.0 * uniform() - 1.0;
		}
		for (int c = 3; c < 7; c++)
			nb += b[c] * b[c];
		if (na < 1e-6 || nb < 1e-6)
			continue;
		pwm::SlerpParams S;
		pwm::slerp_setup(a, b, S);
		const double inv = S.linear ? 0.0 : pwm::dvd(1.0, S.stheta);
		for (int t = 0; t < 8; t++) {
			const double tau = t == 0 ? 0.0 : (t == 1 ? 1.0 : uniform());
			double qp[7], qw[7], Rp[9], Rw[9];
			pwm::interpolate_p(a, b, S, tau, qp);
			pwm::interpolate_w(a, b, S, inv, tau, qw);
			pwm::quat_to_matrix(qp + 3, Rp);
			pwm::quat_to_matrix(qw + 3, Rw);
			interp++;
			bool bad = false;
			for (int c = 0; c < 3; c++)
				bad = bad || pwm::dbits(qp[c]) != pwm::dbits(qw[c]);
			for (int c = 3; c < 7; c++)
				bad = bad || !(__builtin_fabs(qp[c] - qw[c]) < __builtin_ldexp(1.0, -47));
			for (int e = 0; e < 9; e++)
				bad = bad || !(__builtin_fabs(Rp[e] - Rw[e]) < __builtin_ldexp(1.0, -43));
			if (bad)
				mism++;
		}
	}
	printf("mismatches %ld walks %ld jumped %ld tried %ld ties %ld interpolations %ld\n", mism, walks, jumped, tried,
	       ties, interp);
	return mism ? 1 : 0;
}
