// pw_query.cu -- collision-query kernels and their C-ABI entry points.
//
// Replaces the FCL traversal behind UnitWorld::isValid / isDisentangled /
// transitStateToWithContact / isValidTransition / intersectingSegments
// (lib/osr/unit_world.cc:215-264, 405-486, 959-1012; lib/osr/cdmodel.cc:162-229).
//
// Verdict pipeline per query (a state, or one step of a segment):
//   1. FP32 transform of the robot plus a rigorous bound on its deviation from
//      the FP64 transform the oracle uses;
//   2. one warp walks the (env node, robot node) pair tree breadth-first from a
//      shared-memory stack, 32 pairs per iteration, with a separating-axis box
//      test whose slack covers every FP32 error;
//   3. leaf pairs run Moeller's test in FP32 mirroring each FP64 decision
//      (plane signs, axis choice, interval overlap) with forward error bounds:
//      each pair is certified separate, certified intersecting, or uncertain;
//   4. uncertain pairs of queries without a certified hit go to a queue that a
//      second kernel re-tests in FP64 with exactly the oracle's arithmetic.
// A query collides iff a certified hit or an FP64 re-test hit exists, which is
// exactly the FP64 verdict over all triangle pairs.
#include <cub/cub.cuh>

#include <algorithm>
#include <climits>
#include <cstring>
#include <mutex>

#include "pw_internal.cuh"
#include "pw_math.cuh"

namespace {

constexpr int WARPS = 4;                  // warps per block
constexpr int STACK_CAP = 1024;           // node-pair stack entries per warp
constexpr int UNC_CAP = 32;               // uncertain pairs buffered per warp
constexpr float U32 = 5.9604645e-08f;     // 2^-24
constexpr unsigned FULL = 0xffffffffu;
constexpr uint64_t RETEST_CAP = 1u << 22; // queued FP64 re-tests per query batch

// Per-query FP32 transform and error bounds.
struct QF {
	float R[9];
	float AR[9];    // |R| + slack
	float t[3];
	float del;      // bound on |difference of two FP32 vertices - FP64 difference| per coordinate
	float margin;   // absolute slack of every separating-axis test
	float W;        // magnitude bound of any coordinate (scene extent)
};

struct WarpSmem {
	uint2 stack[STACK_CAP];
	uint2 unc[UNC_CAP];
	QF qf[32];
};

// Where the FP64 state of a query comes from when a pair must be re-tested.
struct StateSrc {
	const double *states;      // states kernel: 7 doubles per query
	const double *from, *to;   // segments kernel
	const SegParams *seg;
	const double *ckpt;
};

__device__ __forceinline__ void make_qf(const double *q, const WorldDev &W, QF &o)
{
	const float x = (float)q[4], y = (float)q[5], z = (float)q[6], w = (float)q[3];
	const float tx = 2.f * x, ty = 2.f * y, tz = 2.f * z;
	const float twx = tx * w, twy = ty * w, twz = tz * w;
	const float txx = tx * x, txy = ty * x, txz = tz * x;
	const float tyy = ty * y, tyz = tz * y, tzz = tz * z;
	o.R[0] = 1.f - (tyy + tzz); o.R[1] = txy - twz;         o.R[2] = txz + twy;
	o.R[3] = txy + twz;         o.R[4] = 1.f - (txx + tzz); o.R[5] = tyz - twx;
	o.R[6] = txz - twy;         o.R[7] = tyz + twx;         o.R[8] = 1.f - (txx + tyy);
	o.t[0] = (float)q[0]; o.t[1] = (float)q[1]; o.t[2] = (float)q[2];
	const float s = x * x + y * y + z * z + w * w;
	const float dev = fabsf(1.f - s) + 8.f * U32 * s;
	const float epsR = 16.f * U32 * (1.f + s);
	const float r1 = W.rob.r1;
	const float tinf = fmaxf(fmaxf(fabsf(o.t[0]), fabsf(o.t[1])), fabsf(o.t[2]));
	const float del_r = epsR * r1 + 8.f * U32 * ((1.f + 2.f * s) * r1 + tinf) + 1e-30f;
	const float Wm = tinf + r1 + W.env.emax;
	const float er = epsR + 2.f * dev;
#pragma unroll
	for (int i = 0; i < 9; i++)
		o.AR[i] = fabsf(o.R[i]) + er;
	o.W = Wm;
	o.margin = del_r + er * (3.f * r1 + 4.f * Wm) + 128.f * U32 * Wm;
	o.del = 2.f * fmaxf(del_r, W.del_env);
}

// Separating-axis test of env node box (ca, ea) and robot node box (cb local, eb);
// true when provably disjoint.
__device__ __forceinline__ bool sat_disjoint32(const float4 &A0, const float4 &A1, const float4 &B0,
                                               const float4 &B1, const QF &f)
{
	const float *R = f.R, *AR = f.AR;
	const float T0 = fmaf(R[0], B0.x, fmaf(R[1], B0.y, fmaf(R[2], B0.z, f.t[0]))) - A0.x;
	const float T1 = fmaf(R[3], B0.x, fmaf(R[4], B0.y, fmaf(R[5], B0.z, f.t[1]))) - A0.y;
	const float T2 = fmaf(R[6], B0.x, fmaf(R[7], B0.y, fmaf(R[8], B0.z, f.t[2]))) - A0.z;
	const float ea0 = A1.x, ea1 = A1.y, ea2 = A1.z;
	const float eb0 = B1.x, eb1 = B1.y, eb2 = B1.z;
	const float m = f.margin;
	// env axes
	if (fabsf(T0) > ea0 + fmaf(eb0, AR[0], fmaf(eb1, AR[1], eb2 * AR[2])) + m) return true;
	if (fabsf(T1) > ea1 + fmaf(eb0, AR[3], fmaf(eb1, AR[4], eb2 * AR[5])) + m) return true;
	if (fabsf(T2) > ea2 + fmaf(eb0, AR[6], fmaf(eb1, AR[7], eb2 * AR[8])) + m) return true;
	// robot axes
	if (fabsf(fmaf(T0, R[0], fmaf(T1, R[3], T2 * R[6]))) > fmaf(ea0, AR[0], fmaf(ea1, AR[3], ea2 * AR[6])) + eb0 + m) return true;
	if (fabsf(fmaf(T0, R[1], fmaf(T1, R[4], T2 * R[7]))) > fmaf(ea0, AR[1], fmaf(ea1, AR[4], ea2 * AR[7])) + eb1 + m) return true;
	if (fabsf(fmaf(T0, R[2], fmaf(T1, R[5], T2 * R[8]))) > fmaf(ea0, AR[2], fmaf(ea1, AR[5], ea2 * AR[8])) + eb2 + m) return true;
	// cross axes A_i x B_j
#define PW_CROSS(i1, i2, ti1, ti2, ea_i1, ea_i2, j, j1, j2, eb_j1, eb_j2, i)                                      \
	if (fabsf(ti2 * R[3 * i1 + j] - ti1 * R[3 * i2 + j]) >                                                        \
	    ea_i1 * AR[3 * i2 + j] + ea_i2 * AR[3 * i1 + j] + eb_j1 * AR[3 * i + j2] + eb_j2 * AR[3 * i + j1] + m)   \
		return true;
	PW_CROSS(1, 2, T1, T2, ea1, ea2, 0, 1, 2, eb1, eb2, 0)
	PW_CROSS(1, 2, T1, T2, ea1, ea2, 1, 2, 0, eb2, eb0, 0)
	PW_CROSS(1, 2, T1, T2, ea1, ea2, 2, 0, 1, eb0, eb1, 0)
	PW_CROSS(2, 0, T2, T0, ea2, ea0, 0, 1, 2, eb1, eb2, 1)
	PW_CROSS(2, 0, T2, T0, ea2, ea0, 1, 2, 0, eb2, eb0, 1)
	PW_CROSS(2, 0, T2, T0, ea2, ea0, 2, 0, 1, eb0, eb1, 1)
	PW_CROSS(0, 1, T0, T1, ea0, ea1, 0, 1, 2, eb1, eb2, 2)
	PW_CROSS(0, 1, T0, T1, ea0, ea1, 1, 2, 0, eb2, eb0, 2)
	PW_CROSS(0, 1, T0, T1, ea0, ea1, 2, 0, 1, eb0, eb1, 2)
#undef PW_CROSS
	return false;
}

__device__ __forceinline__ float3 f3sub(float3 a, float3 b) { return make_float3(a.x - b.x, a.y - b.y, a.z - b.z); }
__device__ __forceinline__ float3 f3cross(float3 a, float3 b)
{
	return make_float3(fmaf(a.y, b.z, -a.z * b.y), fmaf(a.z, b.x, -a.x * b.z), fmaf(a.x, b.y, -a.y * b.x));
}
__device__ __forceinline__ float f3dot(float3 a, float3 b) { return fmaf(a.x, b.x, fmaf(a.y, b.y, a.z * b.z)); }
__device__ __forceinline__ float f3inf(float3 a) { return fmaxf(fmaxf(fabsf(a.x), fabsf(a.y)), fabsf(a.z)); }
__device__ __forceinline__ float f3l1(float3 a) { return fabsf(a.x) + fabsf(a.y) + fabsf(a.z); }
__device__ __forceinline__ float f3get(float3 a, int i) { return i == 0 ? a.x : (i == 1 ? a.y : a.z); }

// Plane of S against the vertices of T: signed distances with error bounds.
// D = per-coordinate error of any vertex difference; M = coordinate magnitude.
struct PlaneRes {
	float3 N;
	float etaN;
	float d[3], b[3];
};

__device__ __forceinline__ void plane_bounds(float3 S0, float3 S1, float3 S2, float3 T0, float3 T1, float3 T2,
                                             float D, float M, PlaneRes &r)
{
	const float3 e1 = f3sub(S1, S0), e2 = f3sub(S2, S0);
	r.N = f3cross(e1, e2);
	const float A1 = f3inf(e1), A2 = f3inf(e2);
	const float ee1 = D + U32 * A1, ee2 = D + U32 * A2;
	r.etaN = 2.f * (A1 * ee2 + ee1 * A2 + ee1 * ee2) + 3.f * U32 * A1 * A2;
	const float NL1 = f3l1(r.N) + 3.f * r.etaN;
	const float b64 = 4e-15f * (NL1 + 4.f * A1 * A2) * M;
	const float3 T[3] = { T0, T1, T2 };
#pragma unroll
	for (int k = 0; k < 3; k++) {
		const float3 w = f3sub(T[k], S0);
		const float Wi = f3inf(w), W1 = f3l1(w);
		const float ew = D + U32 * Wi;
		r.d[k] = f3dot(r.N, w);
		r.b[k] = 2.f * (NL1 * ew + r.etaN * (W1 + 3.f * ew) + 3.f * U32 * NL1 * Wi + b64);
	}
}

// -1 / +1 certified sign, 0 uncertain.
__device__ __forceinline__ int csign(float d, float b) { return d > b ? 1 : (d < -b ? -1 : 0); }

// Lone vertex from certified nonzero signs (mirrors the FP64 dispatch).
__device__ __forceinline__ int lone3(const int *s)
{
	if (s[0] * s[1] > 0) return 2;
	if (s[0] * s[2] > 0) return 1;
	return 0;
}

// Interval endpoints on axis `ax` relative to origin O, with an error bound.
__device__ __forceinline__ void interval_bounds(const float *p, const float *d, const float *b, int lone,
                                                float etap, float *lo, float *hi, float *err)
{
	const int o1 = lone == 0 ? 1 : 0;
	const int o2 = lone == 2 ? 1 : 2;
	float e[2], E = 0.f;
	const int oo[2] = { o1, o2 };
#pragma unroll
	for (int k = 0; k < 2; k++) {
		const int o = oo[k];
		const float den = fabsf(d[lone]) + fabsf(d[o]);
		const float bb = b[lone] + b[o];
		const float r = d[lone] / (d[lone] - d[o]);
		const float dr = bb / fmaxf(den - bb, 1e-37f) + 3.f * U32;
		const float pd = p[o] - p[lone];
		e[k] = fmaf(pd, r, p[lone]);
		const float ek = etap + (2.f * etap + U32 * fabsf(pd)) + fabsf(pd) * dr + U32 * (fabsf(p[lone]) + fabsf(pd));
		E = fmaxf(E, ek);
	}
	*lo = fminf(e[0], e[1]);
	*hi = fmaxf(e[0], e[1]);
	*err = E;
}

// FP32 Moeller filter.  0 = certified separate, 1 = certified intersecting, 2 = uncertain.
__device__ __noinline__ int tri_filter(float3 V0, float3 V1, float3 V2, float3 U0, float3 U1, float3 U2, float D,
                                       float M)
{
	PlaneRes pv, pu;
	plane_bounds(V0, V1, V2, U0, U1, U2, D, M, pv);   // du
	int su[3];
#pragma unroll
	for (int k = 0; k < 3; k++) su[k] = csign(pv.d[k], pv.b[k]);
	if (su[0] == 0 || su[1] == 0 || su[2] == 0)
		return 2;
	if (su[0] == su[1] && su[0] == su[2])
		return 0;
	plane_bounds(U0, U1, U2, V0, V1, V2, D, M, pu);   // dv
	int sv[3];
#pragma unroll
	for (int k = 0; k < 3; k++) sv[k] = csign(pu.d[k], pu.b[k]);
	if (sv[0] == 0 || sv[1] == 0 || sv[2] == 0)
		return 2;
	if (sv[0] == sv[1] && sv[0] == sv[2])
		return 0;
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
	const float O = f3get(V0, ax);
	const float pvv[3] = { 0.f, f3get(V1, ax) - O, f3get(V2, ax) - O };
	const float puu[3] = { f3get(U0, ax) - O, f3get(U1, ax) - O, f3get(U2, ax) - O };
	const float P = fmaxf(fmaxf(fmaxf(fabsf(pvv[1]), fabsf(pvv[2])), fmaxf(fabsf(puu[0]), fabsf(puu[1]))),
	                      fabsf(puu[2]));
	const float etap = D + U32 * P;
	float vlo, vhi, verr, ulo, uhi, uerr;
	interval_bounds(pvv, pu.d, pu.b, lone3(sv), etap, &vlo, &vhi, &verr);
	interval_bounds(puu, pv.d, pv.b, lone3(su), etap, &ulo, &uhi, &uerr);
	const float B = 2.f * (verr + uerr + 1e-14f * M);
	const float s1 = ulo - vhi, s2 = vlo - uhi;
	if (s1 > B || s2 > B)
		return 0;
	if (s1 < -B && s2 < -B)
		return 1;
	return 2;
}

__device__ __forceinline__ float3 xf(const QF &f, float4 p)
{
	return make_float3(fmaf(f.R[0], p.x, fmaf(f.R[1], p.y, fmaf(f.R[2], p.z, f.t[0]))),
	                   fmaf(f.R[3], p.x, fmaf(f.R[4], p.y, fmaf(f.R[5], p.z, f.t[1]))),
	                   fmaf(f.R[6], p.x, fmaf(f.R[7], p.y, fmaf(f.R[8], p.z, f.t[2]))));
}

__device__ int leaf_test(const WorldDev &W, const QF &f, int es, int rs, uint32_t *et, uint32_t *rt)
{
	const float4 a = __ldg(W.env.triA + es), b = __ldg(W.env.triB + es), c = __ldg(W.env.triC + es);
	const float4 ra = __ldg(W.rob.triA + rs), rb = __ldg(W.rob.triB + rs), rc = __ldg(W.rob.triC + rs);
	*et = (uint32_t)__float_as_int(a.w);
	*rt = (uint32_t)__float_as_int(ra.w);
	return tri_filter(make_float3(a.x, a.y, a.z), make_float3(b.x, b.y, b.z), make_float3(c.x, c.y, c.z),
	                  xf(f, ra), xf(f, rb), xf(f, rc), f.del, f.W);
}

// FP64 re-test of one triangle pair at state q: exactly the oracle's arithmetic.
__device__ __noinline__ bool retest64(const WorldDev &W, const double *q, uint32_t et, uint32_t rt)
{
	double R[9], t[3], U[3][3];
	pwm::state_transform(q, R, t);
	for (int k = 0; k < 3; k++) {
		const int vi = W.rob.F[3 * rt + k];
		const double p[3] = { W.rob.V64[3 * vi], W.rob.V64[3 * vi + 1], W.rob.V64[3 * vi + 2] };
		pwm::xform_point(R, t, p, U[k]);
	}
	const double *V0 = W.env.V64 + 3 * W.env.F[3 * et + 0];
	const double *V1 = W.env.V64 + 3 * W.env.F[3 * et + 1];
	const double *V2 = W.env.V64 + 3 * W.env.F[3 * et + 2];
	return pwm::tri_tri(V0, V1, V2, U[0], U[1], U[2], 0.0) != 0;
}

__device__ __forceinline__ void seg_slerp(const SegParams &P, pwm::SlerpParams &S)
{
	for (int i = 0; i < 4; i++) {
		S.qa[i] = P.qa[i];
		S.qb[i] = P.qb[i];
	}
	S.d = P.d;
	S.theta = P.theta;
	S.stheta = P.stheta;
	S.linear = P.linear;
}

// FP64 state checked at step k of segment s (unit_world.cc:455-470).
__device__ __noinline__ void seg_state64(const StateSrc &src, uint32_t s, uint32_t k, double *q)
{
	const SegParams &P = src.seg[s];
	double delta = src.ckpt[P.ckpt_base + (k >> 5)];
	for (uint32_t j = 0; j < (k & 31u); j++)
		delta = pwm::advance_delta(delta, P.dist, P.step);
	const double tau = pwm::mul(delta, P.inv_dist);
	pwm::SlerpParams S;
	seg_slerp(P, S);
	pwm::interpolate_p(src.from + 7 * (size_t)s, src.to + 7 * (size_t)s, S, tau, q);
}

__device__ __noinline__ bool retest_entry(const WorldDev &W, const StateSrc &src, const RetestEntry &e)
{
	double q[7];
	if (src.states) {
		for (int i = 0; i < 7; i++)
			q[i] = src.states[7 * (size_t)e.query + i];
	} else {
		seg_state64(src, e.query, e.step, q);
	}
	return retest64(W, q, e.env_tri, e.rob_tri);
}

struct LaneStats {
	unsigned long long node = 0, leaf = 0, inl = 0;
};

// Hand the buffered uncertain pairs to the FP64 queue (CAP entries).  When the
// queue is full the pairs are re-tested here; returns true if one of those hit.
template <uint64_t CAP>
__device__ bool flush_unc(const WarpSmem &sm, int nunc, int lane, uint32_t query, uint32_t step,
                          QueryCounters *ctr, RetestEntry *rq, const WorldDev &W, const StateSrc &src,
                          LaneStats &st)
{
	unsigned long long base = 0;
	if (lane == 0)
		base = atomicAdd(&ctr->retest_count, (unsigned long long)nunc);
	base = __shfl_sync(FULL, base, 0);
	bool hit = false;
	if (lane < nunc) {
		RetestEntry e;
		e.query = query;
		e.step = step;
		e.env_tri = sm.unc[lane].x;
		e.rob_tri = sm.unc[lane].y;
		if (base + lane < CAP) {
			rq[base + lane] = e;
		} else {
			st.inl++;
			hit = retest_entry(W, src, e);
		}
	}
	return __any_sync(FULL, hit);
}

// Warp-cooperative traversal of one query; returns true on a certified hit
// (or an inline FP64 hit).  Uncertain pairs of a query without a hit are queued.
template <uint64_t CAP>
__device__ bool traverse(const WorldDev &W, const QF &f, WarpSmem &sm, int lane, int soft_cap, uint32_t query,
                         uint32_t step, QueryCounters *ctr, RetestEntry *rq, const StateSrc &src, LaneStats &st)
{
	const uint32_t ebase = (uint32_t)W.env.leaf_base, rbase = (uint32_t)W.rob.leaf_base;
	const unsigned lt_mask = (1u << lane) - 1u;
	if (lane == 0)
		sm.stack[0] = make_uint2(0u, 0u);
	__syncwarp();
	int top = 1, nunc = 0;
	bool hit = false;
	while (top > 0) {
		int p = min(top, 32);
		const int room = soft_cap - top;
		if (room < p)
			p = max(1, room);
		const bool active = lane < p;
		uint2 pr = make_uint2(0u, 0u);
		if (active)
			pr = sm.stack[top - p + lane];
		__syncwarp();
		top -= p;
		bool push = false, lhit = false, unc = false;
		uint2 c0 = make_uint2(0u, 0u), c1 = make_uint2(0u, 0u), up = make_uint2(0u, 0u);
		if (active) {
			const float4 A0 = __ldg(W.env.nodeA + pr.x), A1 = __ldg(W.env.nodeB + pr.x);
			const float4 B0 = __ldg(W.rob.nodeA + pr.y), B1 = __ldg(W.rob.nodeB + pr.y);
			st.node++;
			if (!sat_disjoint32(A0, A1, B0, B1, f)) {
				const bool la = pr.x >= ebase, lb = pr.y >= rbase;
				if (la && lb) {
					st.leaf++;
					uint32_t et, rt;
					const int r = leaf_test(W, f, (int)(pr.x - ebase), (int)(pr.y - rbase), &et, &rt);
					if (r == 1) {
						lhit = true;
					} else if (r == 2) {
						unc = true;
						up = make_uint2(et, rt);
					}
				} else {
					const bool da = !la && (lb || (A1.x + A1.y + A1.z) >= (B1.x + B1.y + B1.z));
					if (da) {
						c0 = make_uint2((uint32_t)__float_as_int(A0.w), pr.y);
						c1 = make_uint2((uint32_t)__float_as_int(A1.w), pr.y);
					} else {
						c0 = make_uint2(pr.x, (uint32_t)__float_as_int(B0.w));
						c1 = make_uint2(pr.x, (uint32_t)__float_as_int(B1.w));
					}
					push = true;
				}
			}
		}
		if (__any_sync(FULL, lhit)) {
			hit = true;
			break;
		}
		const unsigned um = __ballot_sync(FULL, unc);
		if (um) {
			const int cnt = __popc(um);
			if (nunc + cnt > UNC_CAP) {
				if (flush_unc<CAP>(sm, nunc, lane, query, step, ctr, rq, W, src, st)) {
					hit = true;
					nunc = 0;
					break;
				}
				nunc = 0;
				__syncwarp();
			}
			if (unc)
				sm.unc[nunc + __popc(um & lt_mask)] = up;
			nunc += cnt;
		}
		const unsigned pm = __ballot_sync(FULL, push);
		if (push) {
			const int o = top + 2 * __popc(pm & lt_mask);
			sm.stack[o] = c0;
			sm.stack[o + 1] = c1;
		}
		top += 2 * __popc(pm);
		__syncwarp();
	}
	__syncwarp();
	if (!hit && nunc > 0)
		hit = flush_unc<CAP>(sm, nunc, lane, query, step, ctr, rq, W, src, st);
	__syncwarp();
	return hit;
}

__device__ void flush_stats(QueryCounters *ctr, const LaneStats &st, unsigned long long queries,
                            unsigned long long items, int lane)
{
	unsigned long long a = st.node, b = st.leaf, c = st.inl;
	for (int o = 16; o > 0; o >>= 1) {
		a += __shfl_down_sync(FULL, a, o);
		b += __shfl_down_sync(FULL, b, o);
		c += __shfl_down_sync(FULL, c, o);
	}
	if (lane == 0) {
		atomicAdd(&ctr->stat[STAT_NODE_TESTS], a);
		atomicAdd(&ctr->stat[STAT_LEAF_TESTS], b);
		atomicAdd(&ctr->stat[STAT_INLINE], c);
		atomicAdd(&ctr->stat[STAT_QUERIES], queries);
		atomicAdd(&ctr->stat[STAT_ITEMS], items);
	}
}

// ------------------------------------------------------------------ states

template <uint64_t CAP>
__global__ void __launch_bounds__(WARPS * 32) k_states(WorldDev W, const double *states, int64_t n,
                                                       uint8_t *out, QueryCounters *ctr, RetestEntry *rq,
                                                       int soft_cap)
{
	extern __shared__ __align__(16) unsigned char smem_raw[];
	const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
	WarpSmem &sm = reinterpret_cast<WarpSmem *>(smem_raw)[warp];
	StateSrc src{ states, nullptr, nullptr, nullptr, nullptr };
	LaneStats st;
	unsigned long long queries = 0, items = 0;
	for (;;) {
		unsigned long long base = 0;
		if (lane == 0)
			base = atomicAdd(&ctr->work, 32ull);
		base = __shfl_sync(FULL, base, 0);
		if (base >= (unsigned long long)n)
			break;
		const int cnt = (int)min((unsigned long long)32, (unsigned long long)n - base);
		if (lane < cnt) {
			double q[7];
			for (int i = 0; i < 7; i++)
				q[i] = states[7 * (base + lane) + i];
			make_qf(q, W, sm.qf[lane]);
		}
		__syncwarp();
		for (int j = 0; j < cnt; j++) {
			const QF f = sm.qf[j];
			const bool hit = traverse<CAP>(W, f, sm, lane, soft_cap, (uint32_t)(base + j), 0u, ctr, rq, src, st);
			if (lane == 0)
				out[base + j] = hit ? 0 : 1;
		}
		queries += cnt;
		items++;
		__syncwarp();
	}
	flush_stats(ctr, st, queries, items, lane);
}

template <uint64_t CAP>
__global__ void k_retest(WorldDev W, StateSrc src, uint8_t *valid_out, int32_t *first_out, QueryCounters *ctr,
                         const RetestEntry *rq)
{
	const unsigned long long cnt = min((unsigned long long)CAP, ctr->retest_count);
	unsigned long long hits = 0;
	for (unsigned long long i = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x; i < cnt;
	     i += (unsigned long long)gridDim.x * blockDim.x) {
		const RetestEntry e = rq[i];
		if (retest_entry(W, src, e)) {
			hits++;
			if (valid_out)
				valid_out[e.query] = 0;
			if (first_out)
				atomicMin(&first_out[e.query], (int32_t)e.step);
		}
	}
	if (hits)
		atomicAdd(&ctr->stat[STAT_RETEST_HITS], hits);
	if (blockIdx.x == 0 && threadIdx.x == 0)
		ctr->stat[STAT_RETESTS] = cnt;
}

struct BoxParams {
	double rc[3], rh[3], Re[9], te[3], ec[3], eh[3];
};

__global__ void k_disentangled(BoxParams B, const double *states, int64_t n, uint8_t *out)
{
	for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
		double q[7];
		for (int k = 0; k < 7; k++)
			q[k] = states[7 * i + k];
		out[i] = (uint8_t)pwm::boxes_disjoint(q, B.rc, B.rh, B.Re, B.te, B.ec, B.eh);
	}
}

// ------------------------------------------------------------------ segments

constexpr double MAX_STEPS = 1073741824.0; // 2^30

// Step size of the mode, and whether the reference loop runs at all.
__device__ __forceinline__ double seg_step(double dist, double vdelta, int mode)
{
	if (mode == PW_SEG_TRANSITION) {
		const double h = pwm::dvd(dist, 2.0);
		return h < vdelta ? h : vdelta;
	}
	return vdelta;
}

// Upper bound of checkpoint slots per segment (steps / 32, rounded up).
__global__ void k_seg_bound(const double *from, const double *to, int64_t n, double vdelta, int mode,
                            int64_t *slots)
{
	const int64_t s = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
	if (s >= n)
		return;
	const double dist = pwm::distance(from + 7 * s, to + 7 * s);
	const double step = seg_step(dist, vdelta, mode);
	int64_t k = 0;
	if (!(step >= dist) && dist == dist && step > 0.0 && dist / step <= MAX_STEPS)
		k = (int64_t)(dist / step * (1.0 + 1e-6)) + 2;
	slots[s] = (k + 31) / 32;
}

// Per-segment constants, exact step count and delta checkpoints every 32 steps.
__global__ void k_seg_setup(const double *from, const double *to, int64_t n, double vdelta, int mode,
                            const int64_t *slots, const int64_t *slot_base, SegParams *params, double *ckpt,
                            int32_t *first, uint32_t *keys, uint32_t *vals, QueryCounters *ctr)
{
	const int64_t s = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
	if (s >= n)
		return;
	const double *a = from + 7 * s, *b = to + 7 * s;
	SegParams P;
	const double dist = pwm::distance(a, b);
	const double step = seg_step(dist, vdelta, mode);
	pwm::SlerpParams S;
	pwm::slerp_setup(a, b, S);
	for (int i = 0; i < 4; i++) {
		P.qa[i] = S.qa[i];
		P.qb[i] = S.qb[i];
	}
	P.d = S.d;
	P.theta = S.theta;
	P.stheta = S.stheta;
	P.linear = S.linear;
	P.dist = dist;
	P.inv_dist = pwm::dvd(1.0, dist);
	P.step = step;
	P.ckpt_base = slot_base[s];
	int32_t code = INT_MAX;
	int64_t K = 0;
	if (step >= dist || dist != dist) {
		code = PW_STEP_NONE;
	} else if (!(step > 0.0) || dist / step > MAX_STEPS) {
		code = -3;
	} else {
		double delta = step;
		const int64_t nslots = slots[s];
		while (delta <= dist) {
			if ((K & 31) == 0) {
				if ((K >> 5) >= nslots) {
					// the step bound was too small: never write past this segment's slots
					atomicExch(&ctr->error, 1u);
					code = -3;
					K = 0;
					break;
				}
				ckpt[P.ckpt_base + (K >> 5)] = delta;
			}
			delta = pwm::advance_delta(delta, dist, step);
			K++;
		}
	}
	P.nsteps = (int32_t)K;
	params[s] = P;
	first[s] = code;
	keys[s] = (uint32_t)((K + 31) / 32);
	vals[s] = (uint32_t)s;
}

// Chunk-major work order: round j holds chunk j of every segment with more
// than j chunks (segments sorted by chunk count, descending).  Computes the
// exclusive offsets of the rounds and the total number of work items.
__global__ void __launch_bounds__(1024) k_rounds(const uint32_t *sorted_keys, int64_t n, int64_t *round_off,
                                                 QueryCounters *ctr)
{
	typedef cub::BlockScan<long long, 1024> Scan;
	__shared__ typename Scan::TempStorage tmp;
	__shared__ long long carry;
	const int64_t R = n > 0 ? (int64_t)sorted_keys[0] : 0;
	if (threadIdx.x == 0)
		carry = 0;
	__syncthreads();
	for (int64_t t0 = 0; t0 < R; t0 += 1024) {
		const int64_t j = t0 + threadIdx.x;
		long long size = 0;
		if (j < R) {
			// number of keys > j in the descending array
			int64_t lo = 0, hi = n;
			while (lo < hi) {
				const int64_t mid = (lo + hi) >> 1;
				if ((int64_t)sorted_keys[mid] > j)
					lo = mid + 1;
				else
					hi = mid;
			}
			size = lo;
		}
		long long excl, total;
		Scan(tmp).ExclusiveSum(size, excl, total);
		if (j < R)
			round_off[j] = carry + excl;
		__syncthreads();
		if (threadIdx.x == 0)
			carry += total;
		__syncthreads();
	}
	if (threadIdx.x == 0) {
		round_off[R] = carry;
		ctr->stat[STAT_TOTAL_ITEMS] = (unsigned long long)carry;
	}
}

__global__ void __launch_bounds__(WARPS * 32) k_segments(WorldDev W, StateSrc src, const uint32_t *order,
                                                         const int64_t *round_off, int64_t nrounds, int32_t *first,
                                                         QueryCounters *ctr, RetestEntry *rq, int soft_cap)
{
	extern __shared__ __align__(16) unsigned char smem_raw[];
	const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
	WarpSmem &sm = reinterpret_cast<WarpSmem *>(smem_raw)[warp];
	LaneStats st;
	unsigned long long queries = 0, items = 0;
	const unsigned long long total = ctr->stat[STAT_TOTAL_ITEMS];
	for (;;) {
		unsigned long long item = 0;
		if (lane == 0)
			item = atomicAdd(&ctr->work, 1ull);
		item = __shfl_sync(FULL, item, 0);
		if (item >= total)
			break;
		// round j: largest j with round_off[j] <= item (lane 0 searches, then broadcast)
		int64_t j = 0;
		if (lane == 0) {
			// round_off[0] = 0 <= item < total = round_off[R]; round_off is non-decreasing
			int64_t lo = 0, hi = nrounds;
			while (hi - lo > 1) {
				const int64_t mid = (lo + hi) >> 1;
				if (round_off[mid] <= (int64_t)item)
					lo = mid;
				else
					hi = mid;
			}
			j = lo;
		}
		j = __shfl_sync(FULL, j, 0);
		const uint32_t s = order[item - round_off[j]];
		const SegParams &P = src.seg[s];
		const int32_t K = P.nsteps;
		const int32_t k0 = (int32_t)(j * 32);
		items++;
		const int cnt = min(32, K - k0);
		if (cnt <= 0)
			continue;
		int32_t cur = 0;
		if (lane == 0)
			cur = *(volatile int32_t *)&first[s];
		cur = __shfl_sync(FULL, cur, 0);
		if (cur <= k0)
			continue;
		if (lane < cnt) {
			double delta = src.ckpt[P.ckpt_base + j];
			for (int t = 0; t < lane; t++)
				delta = pwm::advance_delta(delta, P.dist, P.step);
			const double tau = pwm::mul(delta, P.inv_dist);
			pwm::SlerpParams S;
			seg_slerp(P, S);
			double q[7];
			pwm::interpolate_p(src.from + 7 * (size_t)s, src.to + 7 * (size_t)s, S, tau, q);
			make_qf(q, W, sm.qf[lane]);
		}
		__syncwarp();
		for (int kk = 0; kk < cnt; kk++) {
			const int32_t k = k0 + kk;
			if (lane == 0)
				cur = *(volatile int32_t *)&first[s];
			cur = __shfl_sync(FULL, cur, 0);
			if (cur <= k)
				break;
			const QF f = sm.qf[kk];
			queries++;
			const bool hit = traverse<RETEST_CAP>(W, f, sm, lane, soft_cap, s, (uint32_t)k, ctr, rq, src, st);
			if (hit) {
				if (lane == 0)
					atomicMin(&first[s], k);
				break;
			}
		}
		__syncwarp();
	}
	flush_stats(ctr, st, queries, items, lane);
}

// INT_MAX -> PW_STEP_FREE, and the number of isValid calls the sequential
// reference loop makes (first + 1 on contact, every step when free).
__global__ void k_seg_finalize(int32_t *first, const SegParams *params, int64_t n, QueryCounters *ctr)
{
	typedef cub::BlockReduce<unsigned long long, 256> Reduce;
	__shared__ typename Reduce::TempStorage tmp;
	const int64_t s = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
	unsigned long long checks = 0;
	if (s < n) {
		int32_t f = first[s];
		if (f == INT_MAX) {
			f = PW_STEP_FREE;
			first[s] = f;
		}
		if (f >= 0)
			checks = (unsigned long long)f + 1;
		else if (f == PW_STEP_FREE)
			checks = (unsigned long long)params[s].nsteps;
	}
	const unsigned long long tot = Reduce(tmp).Sum(checks);
	if (threadIdx.x == 0 && tot)
		atomicAdd(&ctr->ref_checks, tot);
}

// ------------------------------------------------------------------ intersecting segments

constexpr int ISECT_CAP = 1 << 20;

// One warp enumerates every leaf pair that is not certified separate.
__global__ void k_isect_collect(WorldDev W, QF f, uint2 *cand, unsigned int *ncand, int soft_cap)
{
	extern __shared__ __align__(16) unsigned char smem_raw[];
	const int lane = threadIdx.x & 31;
	WarpSmem &sm = reinterpret_cast<WarpSmem *>(smem_raw)[0];
	const uint32_t ebase = (uint32_t)W.env.leaf_base, rbase = (uint32_t)W.rob.leaf_base;
	const unsigned lt_mask = (1u << lane) - 1u;
	if (lane == 0)
		sm.stack[0] = make_uint2(0u, 0u);
	__syncwarp();
	int top = 1;
	while (top > 0) {
		int p = min(top, 32);
		const int room = soft_cap - top;
		if (room < p)
			p = max(1, room);
		const bool active = lane < p;
		uint2 pr = make_uint2(0u, 0u);
		if (active)
			pr = sm.stack[top - p + lane];
		__syncwarp();
		top -= p;
		bool push = false;
		uint2 c0 = make_uint2(0u, 0u), c1 = make_uint2(0u, 0u);
		if (active) {
			const float4 A0 = __ldg(W.env.nodeA + pr.x), A1 = __ldg(W.env.nodeB + pr.x);
			const float4 B0 = __ldg(W.rob.nodeA + pr.y), B1 = __ldg(W.rob.nodeB + pr.y);
			if (!sat_disjoint32(A0, A1, B0, B1, f)) {
				const bool la = pr.x >= ebase, lb = pr.y >= rbase;
				if (la && lb) {
					uint32_t et, rt;
					const int r = leaf_test(W, f, (int)(pr.x - ebase), (int)(pr.y - rbase), &et, &rt);
					if (r != 0) {
						const unsigned idx = atomicAdd(ncand, 1u);
						if (idx < ISECT_CAP)
							cand[idx] = make_uint2(et, rt);
					}
				} else {
					const bool da = !la && (lb || (A1.x + A1.y + A1.z) >= (B1.x + B1.y + B1.z));
					if (da) {
						c0 = make_uint2((uint32_t)__float_as_int(A0.w), pr.y);
						c1 = make_uint2((uint32_t)__float_as_int(A1.w), pr.y);
					} else {
						c0 = make_uint2(pr.x, (uint32_t)__float_as_int(B0.w));
						c1 = make_uint2(pr.x, (uint32_t)__float_as_int(B1.w));
					}
					push = true;
				}
			}
		}
		const unsigned pm = __ballot_sync(FULL, push);
		if (push) {
			const int o = top + 2 * __popc(pm & lt_mask);
			sm.stack[o] = c0;
			sm.stack[o + 1] = c1;
		}
		top += 2 * __popc(pm);
		__syncwarp();
	}
}

struct IsectRow {
	double b[3], e[3], mag;
	int32_t et, rt, cop, pad;
};

// FP64 verdict of each candidate; hits get Moeller's segment at the 1e-6 snap.
__global__ void k_isect_eval(WorldDev W, const double *q, const uint2 *cand, const unsigned int *ncand,
                             IsectRow *rows, unsigned int *nrows)
{
	const unsigned cnt = min(*ncand, (unsigned)ISECT_CAP);
	for (unsigned i = blockIdx.x * blockDim.x + threadIdx.x; i < cnt; i += gridDim.x * blockDim.x) {
		const uint32_t et = cand[i].x, rt = cand[i].y;
		double R[9], t[3], U[3][3];
		pwm::state_transform(q, R, t);
		for (int k = 0; k < 3; k++) {
			const int vi = W.rob.F[3 * rt + k];
			const double p[3] = { W.rob.V64[3 * vi], W.rob.V64[3 * vi + 1], W.rob.V64[3 * vi + 2] };
			pwm::xform_point(R, t, p, U[k]);
		}
		const double *V0 = W.env.V64 + 3 * W.env.F[3 * et + 0];
		const double *V1 = W.env.V64 + 3 * W.env.F[3 * et + 1];
		const double *V2 = W.env.V64 + 3 * W.env.F[3 * et + 2];
		if (!pwm::tri_tri(V0, V1, V2, U[0], U[1], U[2], 0.0))
			continue;
		IsectRow r;
		int cop = 0;
		pwm::tri_tri_isect(V0, V1, V2, U[0], U[1], U[2], 1e-6, &cop, r.b, r.e);
		const double dx = pwm::sub(r.e[0], r.b[0]), dy = pwm::sub(r.e[1], r.b[1]), dz = pwm::sub(r.e[2], r.b[2]);
		r.mag = pwm::rt(pwm::add(pwm::add(pwm::mul(dx, dx), pwm::mul(dy, dy)), pwm::mul(dz, dz)));
		r.et = (int32_t)et;
		r.rt = (int32_t)rt;
		r.cop = cop;
		r.pad = 0;
		rows[atomicAdd(nrows, 1u)] = r;
	}
}

// ------------------------------------------------------------------ host helpers

size_t warp_smem_bytes() { return sizeof(WarpSmem); }

int soft_cap_of(const pw_world *w)
{
	const int slack = w->dev.env.depth + w->dev.rob.depth + 8;
	return STACK_CAP - slack;
}

int check_ready(pw_world *w, const char *who)
{
	if (!w)
		return pw_fail(PW_ERR_INVALID_ARG, std::string(who) + ": world is NULL");
	if (!w->ready)
		return pw_fail(PW_ERR_NO_MODEL, std::string(who) + ": call load_env/load_robot, scale_to_unit and angle_model first");
	if (soft_cap_of(w) < 64)
		return pw_fail(PW_ERR_INTERNAL, std::string(who) + ": BVH too deep for the traversal stack");
	return PW_OK;
}

int ensure_query_scratch(pw_world *w)
{
	PW_CUDA(w->counters.reserve(sizeof(QueryCounters)));
	PW_CUDA(w->retest.reserve(sizeof(RetestEntry) * RETEST_CAP));
	return PW_OK;
}

int persistent_grid(pw_world *w, const void *kernel, size_t smem)
{
	int per_sm = 0;
	cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, WARPS * 32, smem);
	if (per_sm < 1)
		per_sm = 1;
	return per_sm * (w->num_sms > 0 ? w->num_sms : 1);
}

// Event i (0: before the traversal, 1: between traversal and re-test, 2: after) on stream st.
int mark(pw_world *w, int i, cudaStream_t st)
{
	if (!w->ev[i])
		PW_CUDA(cudaEventCreate(&w->ev[i]));
	PW_CUDA(cudaEventRecord(w->ev[i], st));
	return PW_OK;
}

int set_smem_attr(const void *kernel, size_t smem)
{
	PW_CUDA(cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
	return PW_OK;
}

} // namespace

// ------------------------------------------------------------------ C ABI

extern "C" int pw_states_valid(pw_world *w, const double *states, int64_t n, uint8_t *valid, void *stream)
{
	int rc = check_ready(w, "pw_states_valid");
	if (rc)
		return rc;
	if (n < 0 || (n > 0 && (!states || !valid)))
		return pw_fail(PW_ERR_INVALID_ARG, "pw_states_valid: bad pointers or size");
	if (n > (int64_t(1) << 32) - 64)
		return pw_fail(PW_ERR_INVALID_ARG, "pw_states_valid: at most 2^32 - 64 states per call");
	PW_CUDA(cudaSetDevice(w->device));
	cudaStream_t st = (cudaStream_t)stream;
	w->last_stream = st;
	rc = ensure_query_scratch(w);
	if (rc)
		return rc;
	QueryCounters *ctr = (QueryCounters *)w->counters.ptr;
	w->timed = false;
	PW_CUDA(cudaMemsetAsync(ctr, 0, sizeof(QueryCounters), st));
	if (n == 0)
		return PW_OK;
	w->last_states = n;
	if (w->dev.env.ntri == 0 || w->dev.rob.ntri == 0) {
		PW_CUDA(cudaMemsetAsync(valid, 1, (size_t)n, st));
		return PW_OK;
	}
	const size_t smem = warp_smem_bytes() * WARPS;
	rc = set_smem_attr((const void *)k_states<RETEST_CAP>, smem);
	if (rc)
		return rc;
	const int grid = persistent_grid(w, (const void *)k_states<RETEST_CAP>, smem);
	RetestEntry *rq = (RetestEntry *)w->retest.ptr;
	rc = mark(w, 0, st);
	if (rc)
		return rc;
	k_states<RETEST_CAP><<<grid, WARPS * 32, smem, st>>>(w->dev, states, n, valid, ctr, rq, soft_cap_of(w));
	mark(w, 1, st);
	StateSrc src{ states, nullptr, nullptr, nullptr, nullptr };
	k_retest<RETEST_CAP><<<w->num_sms * 4, 256, 0, st>>>(w->dev, src, valid, nullptr, ctr, rq);
	mark(w, 2, st);
	w->timed = true;
	PW_CUDA(cudaGetLastError());
	return PW_OK;
}

extern "C" int pw_states_disentangled(pw_world *w, const double *states, int64_t n, uint8_t *out, void *stream)
{
	if (!w)
		return pw_fail(PW_ERR_INVALID_ARG, "pw_states_disentangled: world is NULL");
	if (!w->ready)
		return pw_fail(PW_ERR_NO_MODEL, "Pain in the ass: models not loaded");
	if (n < 0 || (n > 0 && (!states || !out)))
		return pw_fail(PW_ERR_INVALID_ARG, "pw_states_disentangled: bad pointers or size");
	if (n == 0)
		return PW_OK;
	PW_CUDA(cudaSetDevice(w->device));
	BoxParams B;
	for (int c = 0; c < 3; c++) {
		B.rc[c] = w->rob_box_c[c];
		B.rh[c] = w->rob_box_h[c];
		B.ec[c] = w->env_box_c[c];
		B.eh[c] = w->env_box_h[c];
		B.te[c] = w->pert_t[c];
	}
	for (int i = 0; i < 9; i++)
		B.Re[i] = w->pertR[i];
	const int64_t blocks = std::min<int64_t>((n + 255) / 256, (int64_t)w->num_sms * 16);
	k_disentangled<<<(unsigned)blocks, 256, 0, (cudaStream_t)stream>>>(B, states, n, out);
	PW_CUDA(cudaGetLastError());
	return PW_OK;
}

template <typename T>
static int grow(DeviceBuffer &b, size_t count)
{
	PW_CUDA(b.reserve(sizeof(T) * (count ? count : 1)));
	return PW_OK;
}

extern "C" int pw_segments_first_contact(pw_world *w, const double *from, const double *to, int64_t n,
                                         double verify_delta, int mode, int32_t *first_step, void *stream)
{
	int rc = check_ready(w, "pw_segments_first_contact");
	if (rc)
		return rc;
	if (n < 0 || (n > 0 && (!from || !to || !first_step)))
		return pw_fail(PW_ERR_INVALID_ARG, "pw_segments_first_contact: bad pointers or size");
	if (mode != PW_SEG_TRANSIT && mode != PW_SEG_TRANSITION)
		return pw_fail(PW_ERR_INVALID_ARG, "pw_segments_first_contact: unknown mode");
	if (!(verify_delta > 0.0) || !(verify_delta < INFINITY))
		return pw_fail(PW_ERR_INVALID_ARG,
		               "pw_segments_first_contact: verify_delta must be finite and > 0 (the reference loop never ends otherwise)");
	if (n > (int64_t(1) << 31) - 1)
		return pw_fail(PW_ERR_INVALID_ARG, "pw_segments_first_contact: at most 2^31 - 1 segments per call");
	PW_CUDA(cudaSetDevice(w->device));
	cudaStream_t st = (cudaStream_t)stream;
	w->last_stream = st;
	rc = ensure_query_scratch(w);
	if (rc)
		return rc;
	QueryCounters *ctr = (QueryCounters *)w->counters.ptr;
	w->timed = false;
	w->last_states = -1;
	PW_CUDA(cudaMemsetAsync(ctr, 0, sizeof(QueryCounters), st));
	if (n == 0)
		return PW_OK;
	// scratch: params, slot bounds/base, keys/vals (x2), cub temp
	if ((rc = grow<SegParams>(w->seg_params, n)) || (rc = grow<int64_t>(w->misc, 2 * n + 2)) ||
	    (rc = grow<uint32_t>(w->seg_keys, n)) || (rc = grow<uint32_t>(w->seg_order, n)) ||
	    (rc = grow<uint32_t>(w->seg_keys2, n)) || (rc = grow<uint32_t>(w->seg_order2, n)))
		return rc;
	int64_t *slots = (int64_t *)w->misc.ptr;
	int64_t *slot_base = slots + n + 1;
	const int B = 256;
	const unsigned G = (unsigned)((n + B - 1) / B);
	k_seg_bound<<<G, B, 0, st>>>(from, to, n, verify_delta, mode, slots);
	PW_CUDA(cudaGetLastError());
	size_t t1 = 0, t2 = 0;
	PW_CUDA(cub::DeviceScan::ExclusiveSum(nullptr, t1, slots, slot_base, (int)(n + 1), st));
	PW_CUDA(cub::DeviceRadixSort::SortPairsDescending(nullptr, t2, (uint32_t *)nullptr, (uint32_t *)nullptr,
	                                                  (uint32_t *)nullptr, (uint32_t *)nullptr, (int)n, 0, 32, st));
	PW_CUDA(w->cub_tmp.reserve(std::max(t1, t2)));
	// slots[n] = 0 so that slot_base[n] is the total
	PW_CUDA(cudaMemsetAsync(slots + n, 0, sizeof(int64_t), st));
	PW_CUDA(cub::DeviceScan::ExclusiveSum(w->cub_tmp.ptr, t1, slots, slot_base, (int)(n + 1), st));
	// the checkpoint array needs the total: read it back (one small synchronous copy)
	int64_t total_slots = 0;
	PW_CUDA(cudaMemcpyAsync(&total_slots, slot_base + n, sizeof(int64_t), cudaMemcpyDeviceToHost, st));
	PW_CUDA(cudaStreamSynchronize(st));
	if ((rc = grow<double>(w->seg_ckpt, (size_t)total_slots + 1)))
		return rc;
	SegParams *params = (SegParams *)w->seg_params.ptr;
	double *ckpt = (double *)w->seg_ckpt.ptr;
	uint32_t *keys = (uint32_t *)w->seg_keys.ptr, *vals = (uint32_t *)w->seg_order.ptr;
	uint32_t *keys2 = (uint32_t *)w->seg_keys2.ptr, *vals2 = (uint32_t *)w->seg_order2.ptr;
	k_seg_setup<<<G, B, 0, st>>>(from, to, n, verify_delta, mode, slots, slot_base, params, ckpt, first_step, keys,
	                             vals, ctr);
	PW_CUDA(cudaGetLastError());
	PW_CUDA(cub::DeviceRadixSort::SortPairsDescending(w->cub_tmp.ptr, t2, keys, keys2, vals, vals2, (int)n, 0, 32, st));
	// rounds: at most max(slots) + 1 offsets
	int64_t max_rounds = 0;
	{
		// bound the round count by the largest slot bound (copy of the sorted maximum needs the sort;
		// use the slot total as a safe bound when it is small, else read the maximum back)
		uint32_t mx = 0;
		PW_CUDA(cudaMemcpyAsync(&mx, keys2, sizeof(uint32_t), cudaMemcpyDeviceToHost, st));
		PW_CUDA(cudaStreamSynchronize(st));
		max_rounds = mx;
	}
	if ((rc = grow<int64_t>(w->round_off, (size_t)max_rounds + 2)))
		return rc;
	int64_t *round_off = (int64_t *)w->round_off.ptr;
	k_rounds<<<1, 1024, 0, st>>>(keys2, n, round_off, ctr);
	PW_CUDA(cudaGetLastError());
	const size_t smem = warp_smem_bytes() * WARPS;
	rc = set_smem_attr((const void *)k_segments, smem);
	if (rc)
		return rc;
	const int grid = persistent_grid(w, (const void *)k_segments, smem);
	RetestEntry *rq = (RetestEntry *)w->retest.ptr;
	StateSrc src{ nullptr, from, to, params, ckpt };
	rc = mark(w, 0, st);
	if (rc)
		return rc;
	k_segments<<<grid, WARPS * 32, smem, st>>>(w->dev, src, vals2, round_off, max_rounds, first_step, ctr, rq,
	                                           soft_cap_of(w));
	mark(w, 1, st);
	k_retest<RETEST_CAP><<<w->num_sms * 4, 256, 0, st>>>(w->dev, src, nullptr, first_step, ctr, rq);
	mark(w, 2, st);
	w->timed = true;
	k_seg_finalize<<<G, B, 0, st>>>(first_step, params, n, ctr);
	PW_CUDA(cudaGetLastError());
	return PW_OK;
}

extern "C" int pw_intersecting_segments(pw_world *w, const double q[7], int64_t capacity, double *begins,
                                        double *ends, double *mags, int32_t *face_pairs, int32_t *coplanar,
                                        int64_t *count)
{
	int rc = check_ready(w, "pw_intersecting_segments");
	if (rc)
		return rc;
	if (!q || !count || capacity < 0 || (capacity > 0 && (!begins || !ends || !mags || !face_pairs)))
		return pw_fail(PW_ERR_INVALID_ARG, "pw_intersecting_segments: bad argument");
	*count = 0;
	if (w->dev.env.ntri == 0 || w->dev.rob.ntri == 0)
		return PW_OK;
	PW_CUDA(cudaSetDevice(w->device));
	DeviceBuffer dq, dcand, dn, drows;
	PW_CUDA(dq.reserve(sizeof(double) * 7));
	PW_CUDA(dcand.reserve(sizeof(uint2) * ISECT_CAP));
	PW_CUDA(dn.reserve(sizeof(unsigned int) * 2));
	PW_CUDA(drows.reserve(sizeof(IsectRow) * ISECT_CAP));
	PW_CUDA(cudaMemcpy(dq.ptr, q, sizeof(double) * 7, cudaMemcpyHostToDevice));
	PW_CUDA(cudaMemset(dn.ptr, 0, sizeof(unsigned int) * 2));
	QF f;
	{
		// the same FP32 set-up the kernels use, evaluated on the host
		const float x = (float)q[4], y = (float)q[5], z = (float)q[6], ww = (float)q[3];
		const float tx = 2.f * x, ty = 2.f * y, tz = 2.f * z;
		const float twx = tx * ww, twy = ty * ww, twz = tz * ww;
		const float txx = tx * x, txy = ty * x, txz = tz * x;
		const float tyy = ty * y, tyz = tz * y, tzz = tz * z;
		const float R[9] = { 1.f - (tyy + tzz), txy - twz, txz + twy, txy + twz, 1.f - (txx + tzz), tyz - twx,
		                     txz - twy, tyz + twx, 1.f - (txx + tyy) };
		for (int i = 0; i < 9; i++) f.R[i] = R[i];
		f.t[0] = (float)q[0]; f.t[1] = (float)q[1]; f.t[2] = (float)q[2];
		const float s = x * x + y * y + z * z + ww * ww;
		const float dev = fabsf(1.f - s) + 8.f * U32 * s;
		const float epsR = 16.f * U32 * (1.f + s);
		const float r1 = w->dev.rob.r1;
		const float tinf = std::max(std::max(fabsf(f.t[0]), fabsf(f.t[1])), fabsf(f.t[2]));
		const float del_r = epsR * r1 + 8.f * U32 * ((1.f + 2.f * s) * r1 + tinf) + 1e-30f;
		const float Wm = tinf + r1 + w->dev.env.emax;
		const float er = epsR + 2.f * dev;
		for (int i = 0; i < 9; i++) f.AR[i] = fabsf(f.R[i]) + er;
		f.W = Wm;
		// a wider slack on the host side costs nothing here and covers host/device rounding differences
		f.margin = 2.f * (del_r + er * (3.f * r1 + 4.f * Wm) + 128.f * U32 * Wm);
		f.del = 4.f * std::max(del_r, w->dev.del_env);
	}
	const size_t smem = warp_smem_bytes();
	rc = set_smem_attr((const void *)k_isect_collect, smem);
	if (rc)
		return rc;
	unsigned int *ncand = (unsigned int *)dn.ptr;
	k_isect_collect<<<1, 32, smem>>>(w->dev, f, (uint2 *)dcand.ptr, ncand, soft_cap_of(w));
	k_isect_eval<<<w->num_sms, 256>>>(w->dev, (const double *)dq.ptr, (const uint2 *)dcand.ptr, ncand,
	                                  (IsectRow *)drows.ptr, ncand + 1);
	PW_CUDA(cudaGetLastError());
	unsigned int nn[2];
	PW_CUDA(cudaMemcpy(nn, dn.ptr, sizeof(nn), cudaMemcpyDeviceToHost));
	if (nn[0] > (unsigned)ISECT_CAP)
		return pw_fail(PW_ERR_CAPACITY, "pw_intersecting_segments: more than 2^20 candidate pairs");
	std::vector<IsectRow> rows(nn[1]);
	if (nn[1])
		PW_CUDA(cudaMemcpy(rows.data(), drows.ptr, sizeof(IsectRow) * nn[1], cudaMemcpyDeviceToHost));
	std::sort(rows.begin(), rows.end(), [](const IsectRow &a, const IsectRow &b) {
		return a.et != b.et ? a.et < b.et : a.rt < b.rt;
	});
	*count = (int64_t)rows.size();
	const int64_t m = std::min<int64_t>(capacity, *count);
	for (int64_t i = 0; i < m; i++) {
		for (int c = 0; c < 3; c++) {
			begins[3 * i + c] = rows[i].b[c];
			ends[3 * i + c] = rows[i].e[c];
		}
		mags[i] = rows[i].mag;
		face_pairs[2 * i] = rows[i].et;
		face_pairs[2 * i + 1] = rows[i].rt;
		if (coplanar)
			coplanar[i] = rows[i].cop;
	}
	if (capacity < *count)
		return pw_fail(PW_ERR_CAPACITY, "pw_intersecting_segments: capacity smaller than the pair count");
	return PW_OK;
}

extern "C" int pw_world_last_stats(pw_world *w, pw_query_stats *out)
{
	if (!w || !out)
		return pw_fail(PW_ERR_INVALID_ARG, "pw_world_last_stats: NULL argument");
	memset(out, 0, sizeof(*out));
	if (!w->counters.ptr)
		return PW_OK;
	PW_CUDA(cudaSetDevice(w->device));
	PW_CUDA(cudaStreamSynchronize(w->last_stream));
	QueryCounters c;
	PW_CUDA(cudaMemcpy(&c, w->counters.ptr, sizeof(c), cudaMemcpyDeviceToHost));
	out->queries = (int64_t)c.stat[STAT_QUERIES];
	out->node_tests = (int64_t)c.stat[STAT_NODE_TESTS];
	out->leaf_tests = (int64_t)c.stat[STAT_LEAF_TESTS];
	out->retests = (int64_t)c.stat[STAT_RETESTS];
	out->retest_hits = (int64_t)c.stat[STAT_RETEST_HITS];
	out->inline_retests = (int64_t)c.stat[STAT_INLINE];
	out->work_items = (int64_t)c.stat[STAT_ITEMS];
	out->reference_checks = w->last_states >= 0 ? w->last_states : (int64_t)c.ref_checks;
	if (w->timed) {
		float a = 0.f, b = 0.f;
		PW_CUDA(cudaEventElapsedTime(&a, w->ev[0], w->ev[1]));
		PW_CUDA(cudaEventElapsedTime(&b, w->ev[1], w->ev[2]));
		out->traverse_ms = a;
		out->retest_ms = b;
	}
	return PW_OK;
}

// ------------------------------------------------------------------ allocation-free variant
//
// Some callers must not allocate device memory once they are running: a planner
// or simulator that embeds this library inside a framework whose pool allocator
// owns the whole device heap, or a latency-critical loop that cannot afford the
// implicit device synchronisation of cudaMalloc/cudaFree.  For them,
// pw_states_valid_noalloc keeps its scratch (query counters and the FP64
// re-test queue) in the fixed device array below instead of the world's
// buffers.  The array is part of the library image: every GPU that loads the
// library holds it (NOALLOC_BYTES, about 16 MiB) until the process exits.

namespace {
constexpr uint64_t NOALLOC_RETEST_CAP = uint64_t(1) << 20;   // queued FP64 re-tests
constexpr int64_t NOALLOC_MAX_STATES = int64_t(1) << 20;     // states per call
constexpr size_t NOALLOC_CTR_BYTES = 256;                     // QueryCounters, padded
static_assert(sizeof(QueryCounters) <= NOALLOC_CTR_BYTES, "counters do not fit their slot");
constexpr size_t NOALLOC_BYTES = NOALLOC_CTR_BYTES + sizeof(RetestEntry) * NOALLOC_RETEST_CAP;
} // namespace

static __device__ __align__(256) unsigned char g_noalloc_scratch[NOALLOC_BYTES];

// Host code cannot use the name g_noalloc_scratch as a device address; the real
// address is looked up once per device, with that device current.
static std::mutex g_noalloc_mu;
static void *g_noalloc_ptr[128];

static int noalloc_scratch(int device, void **out)
{
	if (device < 0 || device >= 128)
		return pw_fail(PW_ERR_INVALID_ARG, "pw_states_valid_noalloc: device ordinal out of range");
	std::lock_guard<std::mutex> lock(g_noalloc_mu);
	if (!g_noalloc_ptr[device]) {
		void *p = nullptr;
		const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
		if (e != cudaSuccess)
			return pw_cuda_fail(e, "pw_states_valid_noalloc: cudaGetSymbolAddress");
		g_noalloc_ptr[device] = p;
	}
	*out = g_noalloc_ptr[device];
	return PW_OK;
}

extern "C" int pw_states_valid_noalloc(pw_world *w, const double *states, int64_t n, uint8_t *valid, void *stream)
{
	int rc = check_ready(w, "pw_states_valid_noalloc");
	if (rc)
		return rc;
	if (n < 0 || (n > 0 && (!states || !valid)))
		return pw_fail(PW_ERR_INVALID_ARG, "pw_states_valid_noalloc: bad pointers or size");
	if (n > NOALLOC_MAX_STATES)
		return pw_fail(PW_ERR_INVALID_ARG,
		               "pw_states_valid_noalloc: at most 1048576 states per call (split the batch or use "
		               "pw_states_valid)");
	PW_CUDA(cudaSetDevice(w->device));
	void *scratch = nullptr;
	rc = noalloc_scratch(w->device, &scratch);
	if (rc)
		return rc;
	cudaStream_t st = (cudaStream_t)stream;
	QueryCounters *ctr = (QueryCounters *)scratch;
	RetestEntry *rq = (RetestEntry *)((unsigned char *)scratch + NOALLOC_CTR_BYTES);
	// the array keeps the previous call's contents: the counters must start at zero
	PW_CUDA(cudaMemsetAsync(ctr, 0, sizeof(QueryCounters), st));
	if (n == 0)
		return PW_OK;
	if (w->dev.env.ntri == 0 || w->dev.rob.ntri == 0) {
		PW_CUDA(cudaMemsetAsync(valid, 1, (size_t)n, st));
		return PW_OK;
	}
	const size_t smem = warp_smem_bytes() * WARPS;
	rc = set_smem_attr((const void *)k_states<NOALLOC_RETEST_CAP>, smem);
	if (rc)
		return rc;
	const int grid = persistent_grid(w, (const void *)k_states<NOALLOC_RETEST_CAP>, smem);
	k_states<NOALLOC_RETEST_CAP><<<grid, WARPS * 32, smem, st>>>(w->dev, states, n, valid, ctr, rq, soft_cap_of(w));
	StateSrc src{ states, nullptr, nullptr, nullptr, nullptr };
	k_retest<NOALLOC_RETEST_CAP><<<w->num_sms * 4, 256, 0, st>>>(w->dev, src, valid, nullptr, ctr, rq);
	PW_CUDA(cudaGetLastError());
	return PW_OK;
}
