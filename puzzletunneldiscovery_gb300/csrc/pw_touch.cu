// pw_touch.cu -- the result tuple of UnitWorld::transitStateToWithContact
// (lib/osr/unit_world.cc:405-474) for a batch of segments, from their
// first-contact codes.  This is what the touch-configuration sampler
// (src/GP/pipeline/touchq_util.py:8-27, calc_touch) consumes: the last free
// state, the first colliding state (or the last state), `done`, and the two
// taus, for thousands of random segments from one root.
#include <cuda_runtime.h>

#include "pw_internal.cuh"
#include "pw_math.cuh"

namespace {

// One thread per segment.  The taus come from the reference's delta loop
// restated in FP64 (advance_delta), so states are bit-identical to
// pw_segment_step_state and to the oracle.
__global__ void k_contact_states(const double *from, const double *to, const int32_t *first, int64_t n,
                                 double verify_delta, double *last_free, double *contact, uint8_t *done,
                                 float *last_tau, float *tau, int *err)
{
	const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
	if (i >= n)
		return;
	const double *a = from + 7 * i, *b = to + 7 * i;
	double *lf = last_free + 7 * i, *st = contact + 7 * i;
	const double dist = pwm::distance(a, b);
	if (verify_delta >= dist) {
		// unit_world.cc:445-447: nothing checked, the target returned
		for (int c = 0; c < 7; c++) {
			lf[c] = a[c];
			st[c] = b[c];
		}
		done[i] = 0;
		last_tau[i] = 0.f;
		tau[i] = 1.f;
		return;
	}
	if (dist != dist) {
		for (int c = 0; c < 7; c++)
			lf[c] = st[c] = a[c];
		done[i] = 0;
		last_tau[i] = tau[i] = 0.f;
		return;
	}
	const int32_t k = first[i];
	if (k < -1) {
		// PW_STEP_INVALID (or a code that does not belong to this delta)
		atomicCAS(err, 0, 1);
		for (int c = 0; c < 7; c++)
			lf[c] = st[c] = a[c];
		done[i] = 0;
		last_tau[i] = tau[i] = 0.f;
		return;
	}
	const double inv = pwm::dvd(1.0, dist);
	pwm::SlerpParams P;
	pwm::slerp_setup(a, b, P);
	// delta of step j is the value after j updates of the loop (step 0: verify_delta)
	double prev = 0.0, delta = verify_delta;
	if (k >= 0) {
		if (k > 0) {
			prev = pwm::walk_delta(delta, dist, verify_delta, k - 1);
			delta = pwm::advance_delta(prev, dist, verify_delta);
		}
		const double t = pwm::mul(delta, inv);
		pwm::interpolate_p(a, b, P, t, st);
		tau[i] = (float)t;
		if (k == 0) {
			for (int c = 0; c < 7; c++)
				lf[c] = a[c];
			last_tau[i] = 0.f;
		} else {
			const double lt = pwm::mul(prev, inv);
			pwm::interpolate_p(a, b, P, lt, lf);
			last_tau[i] = (float)lt;
		}
		done[i] = 0;
		return;
	}
	// every step free: the last state the loop checked, done = true, outer tau 0
	while (true) {
		// runs of updates that stay at or below dist, taken at once (walk_delta's rule)
		double c;
		const int jump = pwm::delta_jump(delta, dist, verify_delta, 1 << 30, &c);
		if (jump > 0) {
			delta = pwm::add(delta, pwm::mul((double)jump, c));
			continue;
		}
		const double next = pwm::advance_delta(delta, dist, verify_delta);
		if (!(next <= dist))
			break;
		delta = next;
	}
	const double lt = pwm::mul(delta, inv);
	pwm::interpolate_p(a, b, P, lt, lf);
	for (int c = 0; c < 7; c++)
		st[c] = lf[c];
	done[i] = 1;
	last_tau[i] = (float)lt;
	tau[i] = 0.f;
}

} // namespace

extern "C" int pw_segments_contact_states(const double *from, const double *to, const int32_t *first_step, int64_t n,
                                          double verify_delta, double *last_free, double *contact, uint8_t *done,
                                          float *last_tau, float *tau, int *err_flag, void *stream)
{
	PW_TRACE("pw_segments_contact_states");
	if (n < 0 || (n > 0 && (!from || !to || !first_step || !last_free || !contact || !done || !last_tau || !tau ||
	                        !err_flag)))
		return pw_fail(PW_ERR_INVALID_ARG, "pw_segments_contact_states: bad pointers or size");
	if (!(verify_delta > 0.0))
		return pw_fail(PW_ERR_INVALID_ARG, "pw_segments_contact_states: verify_delta must be > 0");
	if (n == 0)
		return PW_OK;
	cudaStream_t st = (cudaStream_t)stream;
	k_contact_states<<<(unsigned)((n + 127) / 128), 128, 0, st>>>(from, to, first_step, n, verify_delta, last_free,
	                                                               contact, done, last_tau, tau, err_flag);
	PW_CUDA(cudaGetLastError());
	return PW_OK;
}

// ------------------------------------------------------------------ plane crossings of expansions
//
// Narrow-passage search on a plate: root r is expanded to `per_root`
// endpoints (ends[r * per_root + j]).  A candidate crosses the plate if some
// probe point of the robot (robot-local unit frame, e.g. points of a knot's
// centre line) lies on different sides of the plane z = plane_z at the root
// and at the endpoint, and the straight-line crossing point of that probe
// lies within |x|, |y| <= extent.  A collision-free segment with such a
// crossing passes the robot through a hole of the plate.  Geometry only, in
// FP32: it selects candidates; the exact segment query decides whether the
// motion is free.

namespace {

// Probe point p placed by state q, in FP32 (a candidate filter, not a verdict).
__device__ __forceinline__ void place(const double *q, const float *p, float *o)
{
	const float w = (float)q[3], x = (float)q[4], y = (float)q[5], z = (float)q[6];
	const float R[9] = { 1.f - 2.f * (y * y + z * z), 2.f * (x * y - w * z), 2.f * (x * z + w * y),
	                     2.f * (x * y + w * z), 1.f - 2.f * (x * x + z * z), 2.f * (y * z - w * x),
	                     2.f * (x * z - w * y), 2.f * (y * z + w * x), 1.f - 2.f * (x * x + y * y) };
	for (int i = 0; i < 3; i++)
		o[i] = R[3 * i] * p[0] + R[3 * i + 1] * p[1] + R[3 * i + 2] * p[2] + (float)q[i];
}

__global__ void k_expansion_crossings(const double *roots, const double *ends, int64_t n, int per_root,
                                      const double *probes, int nprobe, float plane_z, float extent, uint8_t *out)
{
	__shared__ float sp[3 * 64];
	const int np = min(nprobe, 64);
	for (int k = threadIdx.x; k < 3 * np; k += blockDim.x)
		sp[k] = (float)probes[k];
	__syncthreads();
	const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
	if (i >= n)
		return;
	const double *a = roots + 7 * (i / per_root), *b = ends + 7 * i;
	uint8_t hit = 0;
	for (int k = 0; k < np && !hit; k++) {
		float pa[3], pb[3];
		place(a, sp + 3 * k, pa);
		place(b, sp + 3 * k, pb);
		const float za = pa[2] - plane_z, zb = pb[2] - plane_z;
		if ((za < 0.f) != (zb < 0.f) && za != zb) {
			const float t = za / (za - zb);
			const float x = pa[0] + t * (pb[0] - pa[0]), y = pa[1] + t * (pb[1] - pa[1]);
			hit = fabsf(x) <= extent && fabsf(y) <= extent;
		}
	}
	out[i] = hit;
}

} // namespace

extern "C" int pw_expansion_crossings(const double *roots, const double *ends, int64_t n, int per_root,
                                      const double *probes, int nprobe, double plane_z, double extent, uint8_t *out,
                                      void *stream)
{
	PW_TRACE("pw_expansion_crossings");
	if (n < 0 || per_root <= 0 || nprobe < 0 || nprobe > 64 ||
	    (n > 0 && (!roots || !ends || !out || (nprobe > 0 && !probes))))
		return pw_fail(PW_ERR_INVALID_ARG, "pw_expansion_crossings: bad pointers or sizes (at most 64 probes)");
	if (n == 0)
		return PW_OK;
	k_expansion_crossings<<<(unsigned)((n + 255) / 256), 256, 0, (cudaStream_t)stream>>>(
	    roots, ends, n, per_root, probes, nprobe, (float)plane_z, (float)extent, out);
	PW_CUDA(cudaGetLastError());
	return PW_OK;
}

// ------------------------------------------------------------------ expansions
//
// per_root perturbed copies of each root: translation + N(0, sigma_t^2 I),
// and the rotation by a rotation vector ~ N(0, sigma_rot^2 I) applied on the
// left (as osr::apply does, osr_state.cc:244-259), the result normalised.
// Normals from a counter-based generator (SplitMix64 finaliser over
// (seed, candidate, draw)) and the Box-Muller transform with 24-bit uniforms,
// so a (seed, index) pair always gives the same candidate.

namespace {

__device__ __forceinline__ uint64_t mix64(uint64_t z)
{
	z += 0x9E3779B97F4A7C15ull;
	z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
	z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
	return z ^ (z >> 31);
}

// Two independent N(0, 1) values from one 64-bit draw, in FP32 (sampling
// noise, not a verdict: FP32 keeps the transcendentals off GB300's narrow
// FP64 pipe).
__device__ __forceinline__ void normal2(uint64_t bits, float &a, float &b)
{
	const float u1 = ((float)(uint32_t)(bits >> 40) + 0.5f) * (1.0f / 16777216.0f);   // (0, 1)
	const float u2 = ((float)(uint32_t)((bits >> 16) & 0xFFFFFFu) + 0.5f) * (1.0f / 16777216.0f);
	const float r = sqrtf(-2.0f * logf(u1));
	float s, c;
	sincospif(2.0f * u2, &s, &c);
	a = r * c;
	b = r * s;
}

__global__ void k_expand(const double *roots, int64_t n, int per_root, double sigma_t, double sigma_rot,
                         uint64_t seed, double *out)
{
	const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
	if (i >= n)
		return;
	const double *q = roots + 7 * (i / per_root);
	const uint64_t base = mix64(seed ^ mix64((uint64_t)i));
	float g[6];
	normal2(mix64(base + 1), g[0], g[1]);
	normal2(mix64(base + 2), g[2], g[3]);
	normal2(mix64(base + 3), g[4], g[5]);
	double *o = out + 7 * i;
	for (int c = 0; c < 3; c++)
		o[c] = q[c] + sigma_t * (double)g[c];
	const float sr = (float)sigma_rot;
	const float rx = sr * g[3], ry = sr * g[4], rz = sr * g[5];
	const float ang = sqrtf(rx * rx + ry * ry + rz * rz);
	float w1 = 1.f, x1 = 0.f, y1 = 0.f, z1 = 0.f;
	if (ang > 0.f) {
		float sh, ch;
		sincosf(0.5f * ang, &sh, &ch);
		sh /= ang;
		w1 = ch;
		x1 = rx * sh;
		y1 = ry * sh;
		z1 = rz * sh;
	}
	// the endpoint's rotation in FP32 (it is a random perturbation; the segment query
	// normalises and interpolates it in FP64 from the stored value)
	const float w2 = (float)q[3], x2 = (float)q[4], y2 = (float)q[5], z2 = (float)q[6];
	const float w = w1 * w2 - x1 * x2 - y1 * y2 - z1 * z2;
	const float x = w1 * x2 + x1 * w2 + y1 * z2 - z1 * y2;
	const float y = w1 * y2 - x1 * z2 + y1 * w2 + z1 * x2;
	const float z = w1 * z2 + x1 * y2 - y1 * x2 + z1 * w2;
	const float im = rsqrtf(w * w + x * x + y * y + z * z);
	o[3] = (double)(w * im);
	o[4] = (double)(x * im);
	o[5] = (double)(y * im);
	o[6] = (double)(z * im);
}

} // namespace

extern "C" int pw_expand_states(const double *roots, int64_t nroots, int per_root, double sigma_t, double sigma_rot,
                                uint64_t seed, double *out, void *stream)
{
	PW_TRACE("pw_expand_states");
	if (nroots < 0 || per_root <= 0 || !(sigma_t >= 0.0) || !(sigma_rot >= 0.0) ||
	    (nroots > 0 && (!roots || !out)))
		return pw_fail(PW_ERR_INVALID_ARG, "pw_expand_states: bad pointers, sizes or deviations");
	const int64_t n = nroots * per_root;
	if (n == 0)
		return PW_OK;
	k_expand<<<(unsigned)((n + 255) / 256), 256, 0, (cudaStream_t)stream>>>(roots, n, per_root, sigma_t, sigma_rot,
	                                                                      seed, out);
	PW_CUDA(cudaGetLastError());
	return PW_OK;
}

// ------------------------------------------------------------------ key configurations and touch targets

namespace {

// One thread per (surface pair, spin): the state of pwm::keyconf_state.
__global__ void k_keyconf_states(const double *rp, const double *rn, const double *ep, const double *en, int64_t P,
                                 int64_t A, double margin, const double *hc, const double *hs, int per_pair,
                                 double *out)
{
	const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
	if (i >= P * A)
		return;
	const int64_t p = i / A, a = i - p * A;
	const int64_t k = per_pair ? i : a;
	pwm::keyconf_state(rp + 3 * p, rn + 3 * p, ep + 3 * p, en + 3 * p, margin, hc[k], hs[k], out + 7 * i);
}

// A uniform direction on the unit sphere from two 24-bit uniforms (z uniform in
// (-1, 1), azimuth uniform), in FP32: sampling noise, not a verdict.
__device__ __forceinline__ void unit_direction(uint64_t bits, float d[3])
{
	const float u1 = ((float)(uint32_t)(bits >> 40) + 0.5f) * (1.0f / 16777216.0f);
	const float u2 = ((float)(uint32_t)((bits >> 16) & 0xFFFFFFu) + 0.5f) * (1.0f / 16777216.0f);
	const float z = 1.0f - 2.0f * u1;
	const float r = sqrtf(fmaxf(0.0f, 1.0f - z * z));
	float s, c;
	sincospif(2.0f * u2, &s, &c);
	d[0] = r * c;
	d[1] = r * s;
	d[2] = z;
}

// Row i of a touch batch: the key i / per_key, and the target osr::apply
// (osr_state.cc:244-259) makes of it with a random unit-sphere translation and
// a rotation vector uniform in the ball of radius 2 pi, applied on the left.
__global__ void k_touch_targets(const double *keys, int64_t n, int per_key, uint64_t seed, double *from, double *to)
{
	const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
	if (i >= n)
		return;
	const double *q = keys + 7 * (i / per_key);
	const uint64_t base = mix64(seed ^ mix64((uint64_t)i));
	float tr[3], ax[3];
	unit_direction(mix64(base + 1), tr);
	unit_direction(mix64(base + 2), ax);
	const uint64_t b3 = mix64(base + 3);
	const float u3 = ((float)(uint32_t)(b3 >> 40) + 0.5f) * (1.0f / 16777216.0f);
	// radius of a point uniform in the ball: 2 pi * cbrt(u); half of it for the quaternion
	const float half = 3.14159265f * cbrtf(u3);
	float sh, ch;
	sincosf(half, &sh, &ch);
	const double qa[4] = { (double)ch, (double)(sh * ax[0]), (double)(sh * ax[1]), (double)(sh * ax[2]) };
	double rot[4], r[4];
	const double raw[4] = { q[3], q[4], q[5], q[6] };
	pwm::quat_normalize(raw, rot);
	pwm::quat_mul(qa, rot, r);
	double *f = from + 7 * i, *o = to + 7 * i;
	for (int c = 0; c < 7; c++)
		f[c] = q[c];
	for (int c = 0; c < 3; c++)
		o[c] = pwm::add(q[c], (double)tr[c]);
	pwm::quat_normalize(r, o + 3);
}

} // namespace

extern "C" int pw_keyconf_states(const double *rob_points, const double *rob_normals, const double *env_points,
                                 const double *env_normals, int64_t npairs, double margin, const double *half_cos,
                                 const double *half_sin, int64_t nspins, int per_pair_angles, double *out,
                                 void *stream)
{
	PW_TRACE("pw_keyconf_states");
	if (npairs < 0 || nspins <= 0 || !(margin == margin) ||
	    (npairs > 0 && (!rob_points || !rob_normals || !env_points || !env_normals || !half_cos || !half_sin || !out)))
		return pw_fail(PW_ERR_INVALID_ARG, "pw_keyconf_states: bad pointers or sizes");
	if (npairs > (int64_t(1) << 40) / nspins)
		return pw_fail(PW_ERR_INVALID_ARG, "pw_keyconf_states: too many states");
	const int64_t n = npairs * nspins;
	if (n == 0)
		return PW_OK;
	k_keyconf_states<<<(unsigned)((n + 255) / 256), 256, 0, (cudaStream_t)stream>>>(
	    rob_points, rob_normals, env_points, env_normals, npairs, nspins, margin, half_cos, half_sin,
	    per_pair_angles ? 1 : 0, out);
	PW_CUDA(cudaGetLastError());
	return PW_OK;
}

extern "C" int pw_touch_targets(const double *keys, int64_t nkeys, int per_key, uint64_t seed, double *from,
                                double *to, void *stream)
{
	PW_TRACE("pw_touch_targets");
	if (nkeys < 0 || per_key <= 0 || (nkeys > 0 && (!keys || !from || !to)))
		return pw_fail(PW_ERR_INVALID_ARG, "pw_touch_targets: bad pointers or sizes");
	if (nkeys > (int64_t(1) << 40) / per_key)
		return pw_fail(PW_ERR_INVALID_ARG, "pw_touch_targets: too many segments");
	const int64_t n = nkeys * per_key;
	if (n == 0)
		return PW_OK;
	k_touch_targets<<<(unsigned)((n + 255) / 256), 256, 0, (cudaStream_t)stream>>>(keys, n, per_key, seed, from, to);
	PW_CUDA(cudaGetLastError());
	return PW_OK;
}
