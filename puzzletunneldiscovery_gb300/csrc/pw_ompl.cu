// pw_ompl.cu -- OMPL's discrete motion check for batches of motions.
//
// pyse3ompl's OmplDriver::validateMotionPairs (lib/pyse3ompl/ompldriver.cc:597-621)
// calls SpaceInformation::checkMotion once per pair, with OMPL.app's
// SE3RigidBodyPlanning set up for discrete checking at the puzzle's collision
// resolution (setStateValidityCheckingResolution(cdres), ompldriver.cc:676-677)
// and the translation bounded by the puzzle's volume (:679-685).  OMPL is not
// vendored by the reference (an un-vendored fork of OMPL 1.x); what this file
// restates is OMPL's published algorithm:
//   * SE3StateSpace is R^3 x SO(3), both weights 1.  R^3: Euclidean distance,
//     maximum extent |hi - lo|.  SO(3): arc length acos|<q1, q2>| (0 when
//     |<q1, q2>| > 1 - 1e-9), maximum extent pi / 2.
//   * Each component's longest valid segment is its extent times cdres; the
//     compound space's segment count is the largest component count,
//     nd = max(ceil(d_R3 / lvs_R3), ceil(d_SO3 / lvs_SO3)).
//   * DiscreteMotionValidator::checkMotion(s1, s2): s2 is valid and so is
//     interpolate(s1, s2, k / nd) for k = 1 .. nd - 1.  s1 is assumed valid
//     and not checked.  The order OMPL checks them in does not change the
//     answer.
//   * interpolate: R^3 from + (to - from) t; SO(3) from when the arc length is
//     at most DBL_EPSILON, else (q1 s0 + q2 s1) / sin(theta) with
//     s0 = sin((1 - t) theta), s1 = sin(t theta) negated when <q1, q2> < 0.
// sin and acos are pw_math.cuh's own (a few ulp of libm's), so the states
// generated here equal the oracle's bit for bit.  The validity of a state is
// the engine's exact verdict after translateOMPLStateToUnitState
// (unit_world.cc:689-711), as for validateStates.
//
// The check runs in passes, each over the motions that are still valid: the
// targets, then dyadic levels of k.  With m = nd - 1 and T = floor(log2 m),
// level l holds the odd multiples of 2^(T - l) in 1 .. m, so level 0 is the
// single state k = 2^T, each further level halves the spacing of the states
// checked so far, and levels 0 .. T list every k once.  A motion's verdict is
// the AND of all its states either way; the passes only skip the states of
// motions already known to collide, as the early exit of OMPL's bisection
// order does, and stop at the first level no valid motion has.  In a pass, a
// scan of the per-motion counts numbers the pass's states; they are
// generated, converted to the unit frame and checked window by window, and a
// colliding state clears its motion's verdict.
#include <cub/cub.cuh>

#include <cfloat>
#include <cmath>

#include "pw_internal.cuh"
#include "pw_math.cuh"

namespace {

constexpr double QUAT_NORM_ERROR = 1e-9;   // OMPL's MAX_QUATERNION_NORM_ERROR
constexpr double MAX_SEGMENTS = 2147483647.0;
constexpr int64_t WINDOW = int64_t(1) << 22;   // states generated and checked per pass

struct OmplSpace {
	double lvs_r3, lvs_so3;   // longest valid segments of the two components
};

// Raw dot product of the two rotations, in OMPL's storage order (x, y, z, w).
__device__ __forceinline__ double quat_dot(const double *a, const double *b)
{
	using namespace pwm;
	return add(add(add(mul(a[3], b[3]), mul(a[4], b[4])), mul(a[5], b[5])), mul(a[6], b[6]));
}

__device__ __forceinline__ double arc_length(double dq)
{
	const double a = pwm::dabs(dq);
	return a > 1.0 - QUAT_NORM_ERROR ? 0.0 : pwm::acos01(a);
}

__device__ __forceinline__ bool finite7(const double *q)
{
	bool ok = true;
	for (int c = 0; c < 7; c++)
		ok = ok && isfinite(q[c]);
	return ok;
}

// The passes, and the listing of every state a motion's check looks at.
enum { PASS_ALL = 0, PASS_TARGET = 1, PASS_LEVEL = 2 };

// Per motion: OMPL's segment count nd, and the verdict's starting value (0, and
// nd = 0, for a motion with a non-finite component).
__global__ void k_ompl_counts(const double *from, const double *to, int64_t n, OmplSpace S, int64_t *nd_out,
                              uint8_t *valid, int *too_long)
{
	const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
	if (i >= n)
		return;
	using namespace pwm;
	const double *a = from + 7 * i, *b = to + 7 * i;
	if (!finite7(a) || !finite7(b)) {
		nd_out[i] = 0;
		valid[i] = 0;
		return;
	}
	const double dx = sub(a[0], b[0]), dy = sub(a[1], b[1]), dz = sub(a[2], b[2]);
	const double dr = rt(add(add(mul(dx, dx), mul(dy, dy)), mul(dz, dz)));
	const double ds = arc_length(quat_dot(a, b));
	const double nr = ceil(dvd(dr, S.lvs_r3)), ns = ceil(dvd(ds, S.lvs_so3));
	const double nd = nr > ns ? nr : ns;
	if (nd > MAX_SEGMENTS) {
		atomicOr(too_long, 1);
		nd_out[i] = 0;
		valid[i] = 0;
		return;
	}
	nd_out[i] = (int64_t)nd;
	valid[i] = 1;
}

// Exponent of the spacing of level l's states (-1: the motion has no such level).
__device__ __forceinline__ int level_shift(int64_t nd, int level)
{
	if (nd < 2)
		return -1;
	const int T = 63 - __clzll((unsigned long long)(nd - 1));
	return T - level;
}

// States of a motion in a pass: all of them (the target and k = 1 .. nd - 1), the
// target, or one level's; the last two only while the motion is valid.
__device__ __forceinline__ int64_t pass_count(int pass, int level, int64_t nd, uint8_t valid)
{
	switch (pass) {
	case PASS_ALL: return nd >= 2 ? nd : 1;
	case PASS_TARGET: return valid ? 1 : 0;
	default: {
		const int e = level_shift(nd, level);
		return valid && e >= 0 ? (((nd - 1) >> e) + 1) >> 1 : 0;
	}
	}
}

// Index k of the r-th state of a motion in a pass (0: the target).
__device__ __forceinline__ int64_t pass_index(int pass, int level, int64_t nd, int64_t r)
{
	switch (pass) {
	case PASS_ALL: return r;
	case PASS_TARGET: return 0;
	default: return (2 * r + 1) << level_shift(nd, level);
	}
}

__global__ void k_ompl_pass_counts(const int64_t *nd, const uint8_t *valid, int64_t n, int pass, int level,
                                   int64_t *cnt)
{
	const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
	if (i < n)
		cnt[i] = pass_count(pass, level, nd[i], valid[i]);
}

// The motion that state g of a pass belongs to: the last i with offs[i] <= g, so
// that motions without states in the pass (offs[i] == offs[i + 1]) are skipped.
__device__ __forceinline__ int64_t owner(const int64_t *offs, int64_t n, int64_t g)
{
	int64_t lo = 0, hi = n - 1;
	while (lo < hi) {
		const int64_t mid = (lo + hi + 1) >> 1;
		if (offs[mid] <= g)
			lo = mid;
		else
			hi = mid - 1;
	}
	return lo;
}

// OMPL's SE3 interpolate(a, b, t), OMPL states (x, y, z, qx, qy, qz, qw).
__device__ __forceinline__ void ompl_interpolate(const double *a, const double *b, double t, double *o)
{
	using namespace pwm;
	for (int c = 0; c < 3; c++)
		o[c] = add(a[c], mul(sub(b[c], a[c]), t));
	const double dq = quat_dot(a, b);
	const double theta = arc_length(dq);
	if (theta > DBL_EPSILON) {
		const double d = dvd(1.0, sin_q(theta));
		const double s0 = sin_q(mul(sub(1.0, t), theta));
		double s1 = sin_q(mul(t, theta));
		if (dq < 0.0)
			s1 = -s1;
		for (int c = 3; c < 7; c++)
			o[c] = mul(add(mul(a[c], s0), mul(b[c], s1)), d);
	} else {
		for (int c = 3; c < 7; c++)
			o[c] = a[c];
	}
}

// States [first, first + cnt) of a pass, in the unit frame.
__global__ void k_ompl_states(const double *from, const double *to, int64_t n, const int64_t *nd,
                              const int64_t *offs, int pass, int level, int64_t first, int64_t cnt, pwfr::Frame F,
                              double *out)
{
	for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < cnt; k += (int64_t)gridDim.x * blockDim.x) {
		const int64_t g = first + k;
		const int64_t i = owner(offs, n, g);
		const int64_t j = pass_index(pass, level, nd[i], g - offs[i]);
		const double *a = from + 7 * i, *b = to + 7 * i;
		double s[7];
		if (j == 0) {
			for (int c = 0; c < 7; c++)
				s[c] = b[c];
		} else {
			ompl_interpolate(a, b, pwm::dvd((double)j, (double)nd[i]), s);
		}
		pwfr::ompl_to_unit(F, s, out + 7 * k);
	}
}

// A state that collides clears its motion's verdict.
__global__ void k_ompl_reduce(const uint8_t *state_ok, int64_t first, int64_t cnt, const int64_t *offs, int64_t n,
                              uint8_t *valid)
{
	for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < cnt; k += (int64_t)gridDim.x * blockDim.x)
		if (!state_ok[k])
			valid[owner(offs, n, first + k)] = 0;
}

// The R^3 extent and both longest valid segments, with OMPL's own argument checks
// (RealVectorBounds::check, StateSpace::setLongestValidSegmentFraction, setup).
int ompl_space(const double lo[3], const double hi[3], double cdres, OmplSpace &S, const char *who)
{
	if (!lo || !hi)
		return pw_fail(PW_ERR_INVALID_ARG, std::string(who) + ": bounds are NULL");
	if (!(cdres >= DBL_EPSILON && cdres <= 1.0 - DBL_EPSILON))
		return pw_fail(PW_ERR_INVALID_ARG, std::string(who) + ": the resolution must lie in (0, 1)");
	double e = 0.0;
	for (int c = 0; c < 3; c++) {
		if (!(std::isfinite(lo[c]) && std::isfinite(hi[c]) && lo[c] <= hi[c]))
			return pw_fail(PW_ERR_INVALID_ARG, std::string(who) + ": bounds must be finite with lo <= hi");
		const double d = hi[c] - lo[c];
		e = e + d * d;
	}
	S.lvs_r3 = std::sqrt(e) * cdres;
	S.lvs_so3 = pwm::PIO2_HI * cdres;
	if (!(S.lvs_r3 >= DBL_EPSILON))
		return pw_fail(PW_ERR_INVALID_ARG, std::string(who) + ": the bounds have no extent");
	return PW_OK;
}

int blocks_for(const pw_world *w, int64_t cnt)
{
	const int64_t want = (cnt + 255) / 256;
	const int64_t cap = (int64_t)(w->num_sms > 0 ? w->num_sms : 1) * 16;
	return (int)(want < cap ? (want > 0 ? want : 1) : cap);
}

// Scratch of one call.
struct OmplScratch {
	DeviceBuffer nd, cnt, offs, tmp, flag, states, ok;
};

// OMPL's segment count of every motion and the verdicts' starting values.
int ompl_counts(const double *from, const double *to, int64_t n, const OmplSpace &S, cudaStream_t st,
                OmplScratch &B, uint8_t *valid, const char *who)
{
	PW_CUDA(B.nd.reserve(sizeof(int64_t) * (size_t)n));
	PW_CUDA(B.flag.reserve(sizeof(int)));
	int *flag = (int *)B.flag.ptr;
	PW_CUDA(cudaMemsetAsync(flag, 0, sizeof(int), st));
	k_ompl_counts<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(from, to, n, S, (int64_t *)B.nd.ptr, valid, flag);
	int too_long = 0;
	PW_CUDA(cudaMemcpyAsync(&too_long, flag, sizeof(int), cudaMemcpyDeviceToHost, st));
	PW_CUDA(cudaStreamSynchronize(st));
	if (too_long)
		return pw_fail(PW_ERR_INVALID_ARG, std::string(who) + ": a motion needs more than 2^31 - 1 segments");
	return PW_OK;
}

// A pass's per-motion counts, their scan (B.offs, n + 1 entries) and its total.
int ompl_scan(int64_t n, int pass, int level, const uint8_t *valid, cudaStream_t st, OmplScratch &B, int64_t *total)
{
	PW_CUDA(B.cnt.reserve(sizeof(int64_t) * (size_t)n));
	PW_CUDA(B.offs.reserve(sizeof(int64_t) * (size_t)(n + 1)));
	int64_t *cnt = (int64_t *)B.cnt.ptr, *offs = (int64_t *)B.offs.ptr;
	k_ompl_pass_counts<<<(unsigned)((n + 255) / 256), 256, 0, st>>>((const int64_t *)B.nd.ptr, valid, n, pass, level,
	                                                                 cnt);
	PW_CUDA(cudaMemsetAsync(offs, 0, sizeof(int64_t), st));
	size_t tmp_bytes = 0;
	PW_CUDA(cub::DeviceScan::InclusiveSum(nullptr, tmp_bytes, cnt, offs + 1, n, st));
	PW_CUDA(B.tmp.reserve(tmp_bytes > 0 ? tmp_bytes : 1));
	PW_CUDA(cub::DeviceScan::InclusiveSum(B.tmp.ptr, tmp_bytes, cnt, offs + 1, n, st));
	PW_CUDA(cudaMemcpyAsync(total, offs + n, sizeof(int64_t), cudaMemcpyDeviceToHost, st));
	PW_CUDA(cudaStreamSynchronize(st));
	return PW_OK;
}

// One pass of the check: its states, window by window, clear the verdicts of the
// motions they collide on.  *total = the pass's states; *launches counts the
// kernels of this library it launched.
int ompl_pass(pw_world *w, const double *from, const double *to, int64_t n, int pass, int level, uint8_t *valid,
              cudaStream_t st, OmplScratch &B, int64_t *total, int64_t *launches)
{
	int rc = ompl_scan(n, pass, level, valid, st, B, total);
	if (rc)
		return rc;
	*launches += 1;
	if (*total == 0)
		return PW_OK;
	const int64_t all = *total;
	const int64_t win = all < WINDOW ? all : WINDOW;
	PW_CUDA(B.states.reserve(sizeof(double) * 7 * (size_t)win));
	PW_CUDA(B.ok.reserve((size_t)win));
	const int64_t *nd = (const int64_t *)B.nd.ptr, *offs = (const int64_t *)B.offs.ptr;
	double *states = (double *)B.states.ptr;
	uint8_t *ok = (uint8_t *)B.ok.ptr;
	const pwfr::Frame F = world_frame(w);
	for (int64_t first = 0; first < all; first += win) {
		const int64_t cnt = all - first < win ? all - first : win;
		k_ompl_states<<<blocks_for(w, cnt), 256, 0, st>>>(from, to, n, nd, offs, pass, level, first, cnt, F,
		                                                  states);
		PW_CUDA(cudaGetLastError());
		w->last_launches = 0;
		if ((rc = pw_states_valid(w, states, cnt, ok, (void *)st)))
			return rc;
		k_ompl_reduce<<<blocks_for(w, cnt), 256, 0, st>>>(ok, first, cnt, offs, n, valid);
		PW_CUDA(cudaGetLastError());
		*launches += 2 + w->last_launches;
	}
	return PW_OK;
}

int check_motion_args(pw_world *w, const double *from, const double *to, int64_t n, const void *out,
                      const char *who)
{
	if (!w)
		return pw_fail(PW_ERR_INVALID_ARG, std::string(who) + ": world is NULL");
	if (!w->ready)
		return pw_fail(PW_ERR_NO_MODEL, std::string(who) + ": world not ready");
	if (n < 0 || (n > 0 && (!from || !to || !out)))
		return pw_fail(PW_ERR_INVALID_ARG, std::string(who) + ": bad pointers or size");
	return PW_OK;
}

} // namespace

extern "C" int pw_ompl_check_motions(pw_world *w, const double *from, const double *to, int64_t n,
                                     const double lo[3], const double hi[3], double cdres, uint8_t *valid,
                                     int64_t *states_checked, void *stream)
{
	PW_TRACE("pw_ompl_check_motions");
	const char *who = "pw_ompl_check_motions";
	int rc = check_motion_args(w, from, to, n, valid, who);
	if (rc)
		return rc;
	OmplSpace S;
	if ((rc = ompl_space(lo, hi, cdres, S, who)))
		return rc;
	if (states_checked)
		*states_checked = 0;
	if (n == 0)
		return PW_OK;
	PW_CUDA(cudaSetDevice(w->device));
	cudaStream_t st = (cudaStream_t)stream;
	OmplScratch B;
	if ((rc = ompl_counts(from, to, n, S, st, B, valid, who)))
		return rc;
	int64_t checked = 0, launches = 1, total = 0;
	if ((rc = ompl_pass(w, from, to, n, PASS_TARGET, 0, valid, st, B, &total, &launches)))
		return rc;
	checked += total;
	// levels 0 .. 62 cover every nd below 2^63; the first empty level ends the check
	for (int level = 0; total > 0 && level < 63; level++) {
		if ((rc = ompl_pass(w, from, to, n, PASS_LEVEL, level, valid, st, B, &total, &launches)))
			return rc;
		checked += total;
	}
	// the scratch is freed on return: the batch's work must be done by then
	PW_CUDA(cudaStreamSynchronize(st));
	w->last_launches = launches;
	if (states_checked)
		*states_checked = checked;
	return PW_OK;
}

extern "C" int pw_ompl_motion_states(pw_world *w, const double *from, const double *to, int64_t n,
                                     const double lo[3], const double hi[3], double cdres, int64_t capacity,
                                     double *states, int64_t *offsets, int64_t *total, void *stream)
{
	PW_TRACE("pw_ompl_motion_states");
	const char *who = "pw_ompl_motion_states";
	int rc = check_motion_args(w, from, to, n, states, who);
	if (rc)
		return rc;
	if (!total || capacity < 0)
		return pw_fail(PW_ERR_INVALID_ARG, std::string(who) + ": bad capacity or total");
	OmplSpace S;
	if ((rc = ompl_space(lo, hi, cdres, S, who)))
		return rc;
	*total = 0;
	if (n == 0)
		return PW_OK;
	PW_CUDA(cudaSetDevice(w->device));
	cudaStream_t st = (cudaStream_t)stream;
	OmplScratch B;
	DeviceBuffer valid_buf;
	PW_CUDA(valid_buf.reserve((size_t)n));
	uint8_t *valid = (uint8_t *)valid_buf.ptr;
	if ((rc = ompl_counts(from, to, n, S, st, B, valid, who)))
		return rc;
	if ((rc = ompl_scan(n, PASS_ALL, 0, valid, st, B, total)))
		return rc;
	if (offsets)
		PW_CUDA(cudaMemcpyAsync(offsets, B.offs.ptr, sizeof(int64_t) * (size_t)(n + 1), cudaMemcpyDeviceToDevice,
		                        st));
	if (*total > capacity) {
		PW_CUDA(cudaStreamSynchronize(st));
		return pw_fail(PW_ERR_CAPACITY, std::string(who) + ": more states than the capacity");
	}
	k_ompl_states<<<blocks_for(w, *total), 256, 0, st>>>(from, to, n, (const int64_t *)B.nd.ptr,
	                                                    (const int64_t *)B.offs.ptr, PASS_ALL, 0, 0, *total,
	                                                    world_frame(w), states);
	PW_CUDA(cudaGetLastError());
	PW_CUDA(cudaStreamSynchronize(st));
	return PW_OK;
}
