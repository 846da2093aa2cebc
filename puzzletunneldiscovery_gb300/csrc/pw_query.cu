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
#include <thread>
#include <vector>

#include "pw_internal.cuh"
#include "pw_math.cuh"
#include "pw_filter.cuh"
#include "pw_async.cuh"

namespace {

using namespace pwf;

constexpr int WARPS = 4;                  // warps per block
// node-pair stack entries per warp: 416 keeps a warp's shared memory at 6.8 KB, so
// that 8 blocks of 4 warps (with the 1 KB the runtime reserves per block) fit in
// the SM's 228 KB (measured: 5 blocks with 896 entries, 7 with 512, 8 with 384
// took the 1M-segment step from 336 to 299 ms; 416 gained another 1 % on the plate)
constexpr int STACK_CAP = 416;
constexpr int UNC_CAP = 32;               // uncertain pairs buffered per warp
constexpr unsigned FULL = 0xffffffffu;
constexpr uint64_t RETEST_CAP = 1u << 22; // queued FP64 re-tests per query batch

constexpr int SLOT_SHIFT = 27;                       // stack entry: (env node, robot node | slot << 27)
constexpr uint32_t NODE_MASK = (1u << SLOT_SHIFT) - 1u;

constexpr int LEAFQ_CAP = 64;  // leaf pairs waiting for a 32-wide triangle-filter batch

struct WarpSmem {
	uint2 stack[STACK_CAP];
	uint2 unc[UNC_CAP];
	QFs qf[32];
	uint2 leafq[LEAFQ_CAP];    // (env slot, robot slot) of queued leaf pairs
	uint32_t slot_query[32];   // state or segment index of each slot
	uint32_t slot_step[32];    // segment step of each slot (0 for states)
	uint8_t unc_slot[UNC_CAP];
	uint8_t leafq_slot[LEAFQ_CAP];
};

// Where the FP64 state of a query comes from when a pair must be re-tested.
struct StateSrc {
	const double *states;      // states kernel: 7 doubles per query
	const double *from, *to;   // segments kernel
	const SegParams *seg;
	const double *ckpt;
	const QFs *anchors;        // per chunk: FP32 transform of the anchor step
};

__device__ __forceinline__ void make_qf(const double *q, const WorldDev &W, QFs &o, float state_ulps = 0.f)
{
	pwf::make_qf(q, W.rob.r1, W.env.emax, W.del_env, o, state_ulps);
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
	const double delta = pwm::walk_delta(src.ckpt[P.ckpt_base + (k >> 5)], P.dist, P.step, (int)(k & 31u));
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

// Per-lane counters of one kernel launch.  32-bit (the kernels flush them into the
// 64-bit query counters before they can wrap): 64-bit lane counters cost registers
// the traversal loop needs.
struct LaneStats {
	uint32_t node = 0, leaf = 0, inl = 0;
};

// Queue the buffered uncertain pairs whose slot is not in `skip`.  A pair that does
// not fit the queue (CAP entries) is not dropped silently: the mask of the slots
// that lost a pair is returned, and the caller answers those slots again after the
// traversal with inline FP64 re-tests.  (Keeping the FP64 test out of this loop
// keeps a function call out of the traversal, whose registers it would otherwise
// force to local memory.)
template <uint64_t CAP>
__device__ uint32_t flush_unc(const WarpSmem &sm, int nunc, uint32_t skip, int lane, QueryCounters *ctr,
                              RetestEntry *rq)
{
	const int slot = lane < nunc ? (int)sm.unc_slot[lane] : 0;
	const bool mine = lane < nunc && !((skip >> slot) & 1u);
	const unsigned mm = __ballot_sync(FULL, mine);
	if (!mm)
		return 0u;
	unsigned long long base = 0;
	if (lane == 0)
		base = atomicAdd(&ctr->retest_count, (unsigned long long)__popc(mm));
	base = __shfl_sync(FULL, base, 0);
	bool lost = false;
	if (mine) {
		const unsigned long long idx = base + __popc(mm & ((1u << lane) - 1u));
		if (idx < CAP) {
			RetestEntry e;
			e.query = sm.slot_query[slot];
			e.step = sm.slot_step[slot];
			e.env_tri = sm.unc[lane].x;
			e.rob_tri = sm.unc[lane].y;
			rq[idx] = e;
		} else {
			lost = true;
		}
	}
	return __reduce_or_sync(FULL, lost ? (1u << slot) : 0u);
}

// Inline FP64 re-test of this round's uncertain pairs (at most one per lane):
// the mask of slots found in contact.
__device__ __forceinline__ uint32_t retest_inline(const WorldDev &W, const WarpSmem &sm, const StateSrc &src,
                                                  bool unc, uint2 up, int slot, LaneStats &st)
{
	bool h = false;
	if (unc) {
		st.inl++;
		RetestEntry e;
		e.query = sm.slot_query[slot];
		e.step = sm.slot_step[slot];
		e.env_tri = up.x;
		e.rob_tri = up.y;
		h = retest_entry(W, src, e);
	}
	return __reduce_or_sync(FULL, h ? (1u << slot) : 0u);
}

// Separating-axis test of env node e and robot node r under the slot transform
// Q0..Q3, with axis-aligned node boxes (OBB = false: boxes in each mesh's frame)
// or oriented ones (OBB = true).  Returns the certified separation (> 0) or -1,
// and the two nodes' (centre, left child) and (half-extents, right child).
// All 15 axes are evaluated without branches (sat_sep32's default form).
template <bool OBB>
__device__ __forceinline__ float node_pair_sep(const WorldDev &W, uint32_t e, uint32_t r, const float4 &Q0,
                                               const float4 &Q1, const float4 &Q2, const float4 &Q3, float4 &A0,
                                               float4 &A1, float4 &B0, float4 &B1)
{
	if (OBB) {
		A0 = __ldg(W.env.obbA + e);
		A1 = __ldg(W.env.obbB + e);
		B0 = __ldg(W.rob.obbA + r);
		B1 = __ldg(W.rob.obbB + r);
		return sat_sep32_obb(A0, A1, __ldg(W.env.obbR0 + e), __ldg(W.env.obbR1 + e), __ldg(W.env.obbR2 + e), B0, B1,
		                     __ldg(W.rob.obbR0 + r), __ldg(W.rob.obbR1 + r), __ldg(W.rob.obbR2 + r), Q0, Q1, Q2, Q3);
	}
	A0 = __ldg(W.env.nodeA + e);
	A1 = __ldg(W.env.nodeB + e);
	B0 = __ldg(W.rob.nodeA + r);
	B1 = __ldg(W.rob.nodeB + r);
	return sat_sep32(A0, A1, B0, B1, Q0, Q1, Q2, Q3);
}

// One warp answers up to 32 queries at once (slots = set bits of `open`;
// sm.qf, sm.slot_query and sm.slot_step describe them): every stack entry
// carries its slot, lanes test pairs of any open slot, and a slot closes at its
// first certified contact.  Returns the mask of slots in contact.  Uncertain
// pairs of slots still open at the end go to the FP64 queue.
// INLINE = false: uncertain pairs go to the FP64 queue; the slots that lost a pair
// to a full queue are returned in `ovf`.  INLINE = true (the second pass over such
// slots): every uncertain pair is re-tested in FP64 at once.
template <uint64_t CAP, bool INLINE, bool OBB>
__device__ uint32_t traverse_batch(const WorldDev &W, WarpSmem &sm, int lane, uint32_t open, int soft_cap,
                                   QueryCounters *ctr, RetestEntry *rq, const StateSrc &src, LaneStats &st,
                                   uint32_t &ovf)
{
	const uint32_t ebase = (uint32_t)W.env.leaf_base, rbase = (uint32_t)W.rob.leaf_base;
	const unsigned lt_mask = (1u << lane) - 1u;
	const unsigned gt_mask = ~(lt_mask | (1u << lane));
	const int nroot = __popc(open);
	if ((open >> lane) & 1u)
		sm.stack[nroot - 1 - __popc(open & lt_mask)] = make_uint2(0u, (uint32_t)lane << SLOT_SHIFT);
	__syncwarp();
	int top = nroot, nunc = 0, nleaf = 0;
	uint32_t done = ~open, hit = 0u;

	auto add_unc = [&](bool unc, uint2 up, int slot) {
		unc = unc && !((done >> slot) & 1u);
		if (INLINE) {
			const uint32_t ih = retest_inline(W, sm, src, unc, up, slot, st);
			hit |= ih;
			done |= ih;
			return;
		}
		const unsigned um = __ballot_sync(FULL, unc);
		if (!um)
			return;
		if (nunc + __popc(um) > UNC_CAP) {
			ovf |= flush_unc<CAP>(sm, nunc, done, lane, ctr, rq);
			nunc = 0;
			__syncwarp();
		}
		if (unc) {
			const int o = nunc + __popc(um & lt_mask);
			sm.unc[o] = up;
			sm.unc_slot[o] = (uint8_t)slot;
		}
		nunc += __popc(um);
	};
	auto run_leaves = [&](int k) {
		bool lh = false, lu = false;
		uint2 up = make_uint2(0u, 0u);
		int ls = 0;
		if (lane < k) {
			const int i = nleaf - k + lane;
			const uint2 e = sm.leafq[i];
			ls = sm.leafq_slot[i];
			if (!((done >> ls) & 1u)) {
				st.leaf++;
				const QFs &Q = sm.qf[ls];
				const float4 ta = __ldg(W.env.triA + e.x), tb = __ldg(W.env.triB + e.x), tc = __ldg(W.env.triC + e.x);
				const float4 ra = __ldg(W.rob.triA + e.y), rb = __ldg(W.rob.triB + e.y), rc = __ldg(W.rob.triC + e.y);
				float gap;
				const int r = tri_filter(f3(ta), f3(tb), f3(tc), f3(ra), f3(rb), f3(rc), Q.q[0], Q.q[1], Q.q[2],
				                         Q.q[3], Q.q[4].x, &gap);
				if (r == 1) {
					lh = true;
				} else if (r == 2) {
					lu = true;
					up = make_uint2((uint32_t)__float_as_int(ta.w), (uint32_t)__float_as_int(ra.w));
				}
			}
		}
		nleaf -= k;
		__syncwarp();
		const uint32_t hm = __reduce_or_sync(FULL, lh ? (1u << ls) : 0u);
		hit |= hm;
		done |= hm;
		if (done != FULL)
			add_unc(lu, up, ls);
	};

	while ((top > 0 || nleaf > 0) && done != FULL) {
		if (top == 0) {
			run_leaves(nleaf);
			continue;
		}
		int p = min(top, 32);
		const int room = soft_cap - top;
		if (room < p)
			p = max(1, room);
		bool active = lane < p;
		uint2 pr = make_uint2(0u, 0u);
		if (active)
			pr = sm.stack[top - 1 - lane];
		__syncwarp();
		top -= p;
		const int slot = (int)(pr.y >> SLOT_SHIFT);
		const uint32_t rn = pr.y & NODE_MASK;
		if ((done >> slot) & 1u)
			active = false;
		bool push = false, leaf = false;
		uint2 c0 = make_uint2(0u, 0u), c1 = make_uint2(0u, 0u);
		if (active) {
			float4 A0, A1, B0, B1;
			const QFs &Q = sm.qf[slot];
			st.node++;
			if (!(node_pair_sep<OBB>(W, pr.x, rn, Q.q[0], Q.q[1], Q.q[2], Q.q[3], A0, A1, B0, B1) > 0.f)) {
				const bool la = pr.x >= ebase, lb = rn >= rbase;
				if (la && lb) {
					leaf = true;
					c0 = make_uint2(pr.x - ebase, rn - rbase);
				} else {
					const uint32_t sbits = (uint32_t)slot << SLOT_SHIFT;
					const bool da = !la && (lb || (A1.x + A1.y + A1.z) >= (B1.x + B1.y + B1.z));
					if (da) {
						c0 = make_uint2((uint32_t)__float_as_int(A0.w), pr.y);
						c1 = make_uint2((uint32_t)__float_as_int(A1.w), pr.y);
					} else {
						c0 = make_uint2(pr.x, (uint32_t)__float_as_int(B0.w) | sbits);
						c1 = make_uint2(pr.x, (uint32_t)__float_as_int(B1.w) | sbits);
					}
					push = true;
				}
			}
		}
		const unsigned lm = __ballot_sync(FULL, leaf);
		if (leaf) {
			const int o = nleaf + __popc(lm & lt_mask);
			sm.leafq[o] = c0;
			sm.leafq_slot[o] = (uint8_t)slot;
		}
		nleaf += __popc(lm);
		const unsigned pm = __ballot_sync(FULL, push);
		if (push) {
			// lane 0's children end on top
			const int o = top + 2 * __popc(pm & gt_mask);
			sm.stack[o] = c1;
			sm.stack[o + 1] = c0;
		}
		top += 2 * __popc(pm);
		__syncwarp();
		if (nleaf >= 32)
			run_leaves(32);
	}
	__syncwarp();
	if (!INLINE && nunc > 0 && done != FULL)
		ovf |= flush_unc<CAP>(sm, nunc, done, lane, ctr, rq);
	__syncwarp();
	return hit;
}

// A chunk traversal looks closer at a node pair once the motion inflation of its
// step range exceeds this fraction of the pair's largest half-extent: in phase A
// (anchor frame only; the closer look computes every step's FP64 frame) and in
// phase B (per-step frames; the closer look halves the step range).  Measured on
// 1M interlocking-tori segments: one threshold of 0.5 took 126.8 ms per step,
// 0.12 106.1 ms (node tests 4.93e9 -> 3.16e9), 0.06 112.6 ms (8 % of the chunks
// in phase B); 0.25 / 0.06 104.2 ms, with 0.18-0.35 / 0.06-0.08 within 1 ms.
constexpr float SPLIT_COARSE = 0.25f, SPLIT_FINE = 0.06f;

// Stack entry of a chunk traversal: (env node, robot node | s0 << 22 | s1 << 27),
// the consecutive steps s0..s1 of one segment sharing the node pair.
constexpr int S0_SHIFT = 22, S1_SHIFT = 27;
constexpr uint32_t RNODE_MASK = (1u << S0_SHIFT) - 1u;

__device__ __forceinline__ uint32_t range_bits(int s0, int s1)
{
	return ((uint32_t)s0 << S0_SHIFT) | ((uint32_t)s1 << S1_SHIFT);
}

// FP64 state of step k0 + lane of segment s (delta walked from the chunk's
// checkpoint) reduced to the slot's FP32 transform and bounds.
__device__ __noinline__ void chunk_step_qf(const WorldDev &W, const StateSrc &src, uint32_t s, int64_t ckslot,
                                           int lane, QFs &o)
{
	const SegParams &P = src.seg[s];
	const double delta = pwm::walk_delta(src.ckpt[ckslot], P.dist, P.step, lane);
	const double tau = pwm::mul(delta, P.inv_dist);
	pwm::SlerpParams S;
	seg_slerp(P, S);
	double q[7];
	pwm::interpolate_w(src.from + 7 * (size_t)s, src.to + 7 * (size_t)s, S, P.inv_stheta, tau, q);
	make_qf(q, W, o, 1.f);
}

// Traversal of the steps 0..nopen-1 of one segment chunk of cnt steps (slots =
// steps in order; sm.slot_query / sm.slot_step describe them).  A node pair is
// tested once for a whole range of steps, with one step's transform and the
// slack widened by the motion bound (`motion` per step) to the farthest step of
// the range, so a pair separated from the swept robot node is pruned for the
// whole range at once.
//   Phase A uses only the anchor step's transform (sm.qf[anchor], exact, from
//   the set-up kernel) and never splits a range.  The first pair that needs a
//   finer look (a leaf pair, or motion comparable to the node size) switches
//   the warp to phase B: the FP64 state of every step is computed lane-parallel
//   and ranges split in halves around their middle step down to single steps,
//   which take the per-step leaf tests.
// Returns the lowest step in contact as a one-bit mask (0 when none).
// INLINE and `ovf` as in traverse_batch.
template <uint64_t CAP, bool INLINE, bool OBB>
__device__ uint32_t traverse_chunk(const WorldDev &W, WarpSmem &sm, int lane, int nopen, int cnt, int anchor,
                                   float motion, int soft_cap, QueryCounters *ctr, RetestEntry *rq,
                                   const StateSrc &src, LaneStats &st, uint32_t seg, int64_t ckslot,
                                   uint32_t &ndetailed, uint32_t &ovf)
{
	const uint32_t ebase = (uint32_t)W.env.leaf_base, rbase = (uint32_t)W.rob.leaf_base;
	const unsigned lt_mask = (1u << lane) - 1u;
	const unsigned gt_mask = ~(lt_mask | (1u << lane));
	// start from the world's seed pairs (a partition of the root pair), all steps open;
	// the count comes from a ballot, which the compiler sees as warp-uniform
	int top;
	{
		const bool has = lane < W.nseeds;
		if (has) {
			const uint2 sd = __ldg(W.seeds + lane);
			sm.stack[lane] = make_uint2(sd.x, sd.y | range_bits(0, nopen - 1));
		}
		top = __popc(__ballot_sync(FULL, has));
	}
	__syncwarp();
	int nunc = 0, nleaf = 0;
	bool detailed = false;
	uint32_t done = nopen >= 32 ? 0u : ~((1u << nopen) - 1u), hit = 0u;

	// contact at the steps in hm: keep the lowest; every step from it upwards is settled
	auto settle = [&](uint32_t hm) {
		const uint32_t low = hm & (~hm + 1u);
		if (!hit || low < hit)
			hit = low;
		done |= ~(hit - 1u);
	};
	// buffer the uncertain pairs of this round (at most one per lane), flushing when full
	auto add_unc = [&](bool unc, uint2 up, int slot) {
		unc = unc && !((done >> slot) & 1u);
		if (INLINE) {
			const uint32_t ih = retest_inline(W, sm, src, unc, up, slot, st);
			if (ih)
				settle(ih);
			return;
		}
		const unsigned um = __ballot_sync(FULL, unc);
		if (!um)
			return;
		if (nunc + __popc(um) > UNC_CAP) {
			ovf |= flush_unc<CAP>(sm, nunc, done, lane, ctr, rq);
			nunc = 0;
			__syncwarp();
		}
		if (unc) {
			const int o = nunc + __popc(um & lt_mask);
			sm.unc[o] = up;
			sm.unc_slot[o] = (uint8_t)slot;
		}
		nunc += __popc(um);
	};
	// run the triangle filter on the newest k queued leaf pairs, one per lane
	auto run_leaves = [&](int k) {
		bool lh = false, lu = false;
		uint2 up = make_uint2(0u, 0u);
		int ls = 0;
		if (lane < k) {
			const int i = nleaf - k + lane;
			const uint2 e = sm.leafq[i];
			ls = sm.leafq_slot[i];
			if (!((done >> ls) & 1u)) {
				st.leaf++;
				const QFs &Q = sm.qf[ls];
				const float4 ta = __ldg(W.env.triA + e.x), tb = __ldg(W.env.triB + e.x), tc = __ldg(W.env.triC + e.x);
				const float4 ra = __ldg(W.rob.triA + e.y), rb = __ldg(W.rob.triB + e.y), rc = __ldg(W.rob.triC + e.y);
				float gap;
				const int r = tri_filter(f3(ta), f3(tb), f3(tc), f3(ra), f3(rb), f3(rc), Q.q[0], Q.q[1], Q.q[2],
				                         Q.q[3], Q.q[4].x, &gap);
				if (r == 1) {
					lh = true;
				} else if (r == 2) {
					lu = true;
					up = make_uint2((uint32_t)__float_as_int(ta.w), (uint32_t)__float_as_int(ra.w));
				}
			}
		}
		nleaf -= k;
		__syncwarp();
		const uint32_t hm = __reduce_or_sync(FULL, lh ? (1u << ls) : 0u);
		if (hm)
			settle(hm);
		if (done != FULL)
			add_unc(lu, up, ls);
	};

	while ((top > 0 || nleaf > 0) && done != FULL) {
		if (top == 0) {
			run_leaves(nleaf);
			continue;
		}
		int p = min(top, 32);
		const int room = soft_cap - top;
		if (room < p)
			p = max(1, room);
		bool active = lane < p;
		uint2 pr = make_uint2(0u, 0u);
		if (active)
			pr = sm.stack[top - 1 - lane];
		__syncwarp();
		top -= p;
		const int s0 = (int)((pr.y >> S0_SHIFT) & 31u);
		int s1 = (int)(pr.y >> S1_SHIFT);
		const uint32_t rn = pr.y & RNODE_MASK;
		if (active) {
			// steps from the lowest contact upwards are settled
			const uint32_t above = done >> s0;
			if (above & 1u)
				active = false;
			else if (above)
				s1 = min(s1, s0 + __ffs(above) - 2);
		}
		bool push2 = false, push1 = false, leaf = false, need = false;
		uint2 c0 = make_uint2(0u, 0u), c1 = make_uint2(0u, 0u);
		if (active) {
			float4 A0, A1, B0, B1;
			const int ref = detailed ? (s0 + s1) >> 1 : anchor;
			const int reach = max(abs(s0 - ref), abs(s1 - ref));
			const QFs &Q = sm.qf[ref];
			const float4 Q0 = Q.q[0], Q1 = Q.q[1], Q2 = Q.q[2];
			float4 Q3 = Q.q[3];
			float infl = 0.f;
			if (reach > 0) {
				infl = (float)reach * motion + 1e-9f * (1.f + Q3.w);
				Q3.y += infl;
			}
			st.node++;
			if (!(node_pair_sep<OBB>(W, pr.x, rn, Q0, Q1, Q2, Q3, A0, A1, B0, B1) > 0.f)) {
				const bool la = pr.x >= ebase, lb = rn >= rbase;
				const float ext = fmaxf(fmaxf(fmaxf(A1.x, A1.y), A1.z), fmaxf(fmaxf(B1.x, B1.y), B1.z));
				const bool fine = (la && lb) || infl > (detailed ? SPLIT_FINE : SPLIT_COARSE) * ext;
				if (!detailed && fine) {
					// hand the pair back for phase B
					need = true;
					push1 = true;
					c0 = make_uint2(pr.x, rn | range_bits(s0, s1));
				} else if (s1 > s0 && fine) {
					// split the step range; the lower half ends on top
					c0 = make_uint2(pr.x, rn | range_bits(s0, ref));
					c1 = make_uint2(pr.x, rn | range_bits(ref + 1, s1));
					push2 = true;
				} else if (la && lb) {
					leaf = true;
					c0 = make_uint2(pr.x - ebase, rn - rbase);
				} else {
					const uint32_t rb_ = range_bits(s0, s1);
					const bool da = !la && (lb || (A1.x + A1.y + A1.z) >= (B1.x + B1.y + B1.z));
					if (da) {
						c0 = make_uint2((uint32_t)__float_as_int(A0.w), rn | rb_);
						c1 = make_uint2((uint32_t)__float_as_int(A1.w), rn | rb_);
					} else {
						c0 = make_uint2(pr.x, (uint32_t)__float_as_int(B0.w) | rb_);
						c1 = make_uint2(pr.x, (uint32_t)__float_as_int(B1.w) | rb_);
					}
					push2 = true;
				}
			}
		}
		// queue leaf pairs; filter them 32 at a time
		const unsigned lm = __ballot_sync(FULL, leaf);
		if (leaf) {
			const int o = nleaf + __popc(lm & lt_mask);
			sm.leafq[o] = c0;
			sm.leafq_slot[o] = (uint8_t)s0;
		}
		nleaf += __popc(lm);
		const unsigned pm2 = __ballot_sync(FULL, push2), pm1 = __ballot_sync(FULL, push1);
		// lane 0's entries end on top
		const int o = top + 2 * __popc(pm2 & gt_mask) + __popc(pm1 & gt_mask);
		if (push2) {
			sm.stack[o] = c1;
			sm.stack[o + 1] = c0;
		} else if (push1) {
			sm.stack[o] = c0;
		}
		top += 2 * __popc(pm2) + __popc(pm1);
		if (!detailed && __any_sync(FULL, need)) {
			if (lane < cnt)
				chunk_step_qf(W, src, seg, ckslot, lane, sm.qf[lane]);
			detailed = true;
			ndetailed++;
		}
		__syncwarp();
		if (nleaf >= 32)
			run_leaves(32);
	}
	__syncwarp();
	if (!INLINE && nunc > 0 && done != FULL)
		ovf |= flush_unc<CAP>(sm, nunc, done, lane, ctr, rq);
	__syncwarp();
	return hit;
}

__device__ void flush_stats(QueryCounters *ctr, LaneStats &st, unsigned long long queries,
                            unsigned long long items, int lane)
{
	unsigned long long a = st.node, b = st.leaf, c = st.inl;
	st = LaneStats();
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

// Second pass over the slots of a state batch that lost uncertain pairs to a full
// FP64 queue: the same traversal with every uncertain pair re-tested inline.
// Returns the mask of those slots in contact.  Not inlined: the FP64 code stays out
// of the register allocation of the kernel's main loop.
template <uint64_t CAP, bool OBB>
__device__ __noinline__ uint32_t resolve_states(const WorldDev &W, WarpSmem &sm, int lane, uint32_t open,
                                                int soft_cap, QueryCounters *ctr, RetestEntry *rq,
                                                const StateSrc &src, LaneStats &st)
{
	uint32_t unused = 0;
	return traverse_batch<CAP, true, OBB>(W, sm, lane, open, soft_cap, ctr, rq, src, st, unused);
}

// Lane counters are flushed into the query counters before a 32-bit count can wrap.
__device__ __forceinline__ bool stats_full(const LaneStats &st, int lane)
{
	return __any_sync(FULL, ((st.node | st.leaf | st.inl) >> 30) != 0u);
}

template <uint64_t CAP, bool OBB>
__global__ void __launch_bounds__(WARPS * 32, 8) k_states(WorldDev W, const double *states, int64_t n,
                                                       uint8_t *out, QueryCounters *ctr, RetestEntry *rq,
                                                       int soft_cap, int width)
{
	extern __shared__ __align__(16) unsigned char smem_raw[];
	const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
	WarpSmem &sm = reinterpret_cast<WarpSmem *>(smem_raw)[warp];
	const StateSrc src{ states, nullptr, nullptr, nullptr, nullptr, nullptr };
	LaneStats st;
	unsigned long long queries = 0, items = 0;
	for (;;) {
		unsigned long long base = 0;
		if (lane == 0)
			base = atomicAdd(&ctr->work, (unsigned long long)width);
		base = __shfl_sync(FULL, base, 0);
		if (base >= (unsigned long long)n)
			break;
		const int cnt = (int)min((unsigned long long)width, (unsigned long long)n - base);
		bool finite = true;
		if (lane < cnt) {
			double q[7];
			for (int i = 0; i < 7; i++) {
				q[i] = states[7 * (base + lane) + i];
				finite = finite && isfinite(q[i]);
			}
			make_qf(q, W, sm.qf[lane]);
			sm.slot_query[lane] = (uint32_t)(base + lane);
			sm.slot_step[lane] = 0u;
		}
		// a non-finite state is answered "not free" without a traversal
		const uint32_t bad = __ballot_sync(FULL, !finite);
		if (bad && lane == 0)
			atomicOr(&ctr->error, (unsigned)PW_DEVERR_NONFINITE);
		__syncwarp();
		const uint32_t open = (cnt == 32 ? FULL : ((1u << cnt) - 1u)) & ~bad;
		uint32_t ovf = 0u;
		uint32_t hit = traverse_batch<CAP, false, OBB>(W, sm, lane, open, soft_cap, ctr, rq, src, st, ovf) | bad;
		ovf &= ~hit;
		if (ovf)
			hit |= resolve_states<CAP, OBB>(W, sm, lane, ovf, soft_cap, ctr, rq, src, st);
		if (lane < cnt)
			out[base + lane] = ((hit >> lane) & 1u) ? 0 : 1;
		queries += cnt;
		items++;
		if (stats_full(st, lane))
			flush_stats(ctr, st, 0, 0, lane);
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
	double ce[3];   // Re ec + te (pwm::xform_point, the FP64 test's own placement)
};

// The FP32 test decides almost every state; the undecided ones are queued
// (warp-aggregated) for k_disentangled64.  The queue holds n entries, so it
// cannot fill.  A persistent block takes tiles of 256 states (56 B each, 14 KB)
// round robin: full tiles of a 16-byte aligned batch stream through a ring of
// DIS_STAGES shared-memory stages filled by bulk copies, so the copies of the
// next tiles are in flight while one is tested; the last partial tile (and
// every tile of a batch that is not 16-byte aligned) is read with plain loads.
// Each thread tests two states of a tile (t and t + 128) with packed f32x2
// arithmetic.  A bulk copy that does not land within DIS_WAIT_NS sets
// PW_DEVERR_WAIT; the block then waits (bounded) for its copies in flight and
// stops.
constexpr int DIS_BLOCK = 256;     // states per tile
constexpr int DIS_THREADS = 128;   // threads per block: two states each
constexpr int DIS_STAGES = 3;
constexpr uint32_t DIS_TILE_BYTES = DIS_BLOCK * 7 * sizeof(double);
constexpr size_t DIS_SMEM = DIS_STAGES * (size_t)DIS_TILE_BYTES + DIS_STAGES * sizeof(uint64_t);
constexpr uint64_t DIS_WAIT_NS = 1000000000ull;

// Records one state's FP32 verdict v (has: the state exists); undecided states
// go to the queue (verdict 0 until k_disentangled64 writes it).  All threads of
// the block call it.
__device__ __forceinline__ void dis_record(int v, bool has, int64_t i, int64_t n, uint8_t *out, uint32_t *queue,
                                           QueryCounters *ctr)
{
	const int lane = threadIdx.x & 31;
	const bool undecided = has && v < 0;
	const unsigned m = __ballot_sync(0xffffffffu, undecided);
	unsigned long long base = 0;
	if (m) {
		if (lane == 0)
			base = atomicAdd(&ctr->retest_count, (unsigned long long)__popc(m));
		base = __shfl_sync(0xffffffffu, base, 0);
	}
	if (undecided) {
		const unsigned long long slot = base + __popc(m & ((1u << lane) - 1u));
		if (slot < (unsigned long long)n)
			queue[slot] = (uint32_t)i;
		v = 0;
	}
	if (has)
		out[i] = (uint8_t)v;
}

// The two states of this thread in a tile staged at sq (states b0 .. b0 + cnt - 1).
template <bool ROT>
__device__ __forceinline__ void dis_tile(const pwf::DisBoxes32 &B32, const double *sq, int64_t b0, int cnt, int64_t n,
                                         uint8_t *out, uint32_t *queue, QueryCounters *ctr)
{
	const int ta = threadIdx.x, tb = threadIdx.x + DIS_THREADS;
	int va = 0, vb = 0;
	pwf::boxes_disjoint32x2<ROT>(sq + 7 * ta, sq + 7 * tb, B32, va, vb);
	dis_record(va, ta < cnt, b0 + ta, n, out, queue, ctr);
	dis_record(vb, tb < cnt, b0 + tb, n, out, queue, ctr);
}

// ROT: the perturbation rotation is not exactly the identity.
template <bool ROT>
__global__ void __launch_bounds__(DIS_THREADS) k_disentangled(pwf::DisBoxes32 B32, const double *states, int64_t n,
                                                              uint8_t *out, uint32_t *queue, QueryCounters *ctr)
{
	extern __shared__ __align__(128) unsigned char dis_smem[];
	double *sq = reinterpret_cast<double *>(dis_smem);
	const uint32_t bar0 = pwa::smem_u32(dis_smem + DIS_STAGES * DIS_TILE_BYTES);
	const bool lead = threadIdx.x == 0;
	const int64_t nfull = (((uintptr_t)states) & 15) == 0 ? n / DIS_BLOCK : 0;
	int64_t tile = blockIdx.x;
	if (tile < nfull) {
		const uint32_t sbase = pwa::smem_u32(dis_smem);
		const int64_t stride = gridDim.x;
		auto issue = [&](int s, int64_t t) {
			pwa::mbar_expect_tx(bar0 + 8 * s, DIS_TILE_BYTES);
			pwa::bulk_g2s(sbase + s * DIS_TILE_BYTES, states + t * (DIS_BLOCK * 7), DIS_TILE_BYTES, bar0 + 8 * s);
		};
		__shared__ int stop;
		if (lead) {
			stop = 0;
			for (int s = 0; s < DIS_STAGES; s++)
				pwa::mbar_init(bar0 + 8 * s, 1);
			pwa::fence_mbar_init();
			for (int s = 0; s < DIS_STAGES && tile + s * stride < nfull; s++)
				issue(s, tile + s * stride);
		}
		__syncthreads();
		uint32_t k = 0;
		for (; tile < nfull; tile += stride, k++) {
			const int s = (int)(k % DIS_STAGES);
			const uint32_t parity = (k / DIS_STAGES) & 1u;
			// one thread polls; the others wait at the block barrier, which also orders
			// the landed copy before their reads
			if (lead && !pwa::mbar_wait_for(bar0 + 8 * s, parity, DIS_WAIT_NS))
				stop = 1;
			__syncthreads();
			if (stop)
				break;
			dis_tile<ROT>(B32, sq + (size_t)s * DIS_BLOCK * 7, tile * DIS_BLOCK, DIS_BLOCK, n, out, queue, ctr);
			__syncthreads();   // every thread is done with stage s
			const int64_t next = tile + (int64_t)DIS_STAGES * stride;
			if (lead && next < nfull) {
				pwa::fence_proxy_async();
				issue(s, next);
			}
		}
		if (stop) {
			// the copies still in flight land before the block's shared memory is released
			if (lead) {
				atomicOr(&ctr->error, (unsigned)PW_DEVERR_WAIT);
				for (uint32_t d = 0; d < (uint32_t)DIS_STAGES && tile + d * stride < nfull; d++)
					pwa::mbar_wait_for(bar0 + 8 * ((k + d) % DIS_STAGES), ((k + d) / DIS_STAGES) & 1u, DIS_WAIT_NS);
			}
			return;
		}
		__syncthreads();
	}
	// the partial last tile, or every tile of an unaligned batch
	for (; tile * DIS_BLOCK < n; tile += gridDim.x) {
		const int64_t b0 = tile * DIS_BLOCK;
		const int cnt = (int)min((int64_t)DIS_BLOCK, n - b0);
		const double *src = states + 7 * b0;
		for (int k = threadIdx.x; k < DIS_BLOCK * 7; k += DIS_THREADS)
			sq[k] = k < cnt * 7 ? src[k] : 0.0;
		__syncthreads();
		dis_tile<ROT>(B32, sq, b0, cnt, n, out, queue, ctr);
		__syncthreads();
	}
}

// The FP64 test of the queued states (ROT as for k_disentangled), one thread
// each, in one-warp blocks so that a short queue spreads over every SM (GB300's
// FP64 pipe is narrow: a block of 256 queued states on one SM took several
// times longer than the same states on eight).
constexpr int DIS64_BLOCK = 32;
template <bool ROT>
__global__ void __launch_bounds__(DIS64_BLOCK) k_disentangled64(BoxParams B, const double *states,
                                                                const uint32_t *queue, int64_t n,
                                                                QueryCounters *ctr, uint8_t *out)
{
	const unsigned long long cnt = min(ctr->retest_count, (unsigned long long)n);
	if (blockIdx.x == 0 && threadIdx.x == 0)
		ctr->stat[STAT_RETESTS] = ctr->retest_count;
	for (unsigned long long k = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x; k < cnt;
	     k += (unsigned long long)gridDim.x * blockDim.x) {
		const int64_t i = (int64_t)queue[k];
		double q[7];
		for (int c = 0; c < 7; c++)
			q[c] = states[7 * i + c];
		bool finite = true;
		for (int c = 0; c < 7; c++)
			finite = finite && isfinite(q[c]);
		out[i] = (uint8_t)(ROT || !finite ? pwm::boxes_disjoint_placed<true>(q, B.rc, B.rh, B.Re, B.ce, B.eh)
		                                  : pwm::boxes_disjoint_placed<false>(q, B.rc, B.rh, B.Re, B.ce, B.eh));
	}
}

// The FP32 constants of the box test.
static pwf::DisBoxes32 dis_boxes32(const BoxParams &B)
{
	pwf::DisBoxes32 o;
	float cabs = 0.f;
	for (int c = 0; c < 3; c++) {
		o.rc[c] = (float)B.rc[c];
		o.rh[c] = (float)B.rh[c];
		o.eh[c] = (float)B.eh[c];
		o.ce[c] = (float)B.ce[c];
		cabs = std::max(cabs, std::fabs(o.ce[c]));
	}
	for (int i = 0; i < 9; i++)
		o.Re[i] = (float)B.Re[i];
	o.ce_abs = cabs * (1.f + 1e-6f);
	return o;
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
// Anchor step of a chunk of cnt steps: the middle step of a full chunk.
__device__ __forceinline__ int anchor_of(int cnt) { return cnt >= 16 ? 15 : (cnt - 1) / 2; }

// FP32 transform (QFs) of the step whose delta is given, from its FP64 state.
__device__ __forceinline__ void seg_step_qf(const WorldDev &W, const double *a, const double *b, const SegParams &P,
                                            double delta, QFs &o)
{
	const double tau = pwm::mul(delta, P.inv_dist);
	pwm::SlerpParams S;
	seg_slerp(P, S);
	double q[7];
	pwm::interpolate_w(a, b, S, P.inv_stheta, tau, q);
	make_qf(q, W, o, 1.f);
}

// First round of each phase of a segment query (the last phase is open), and
// the fewest 32-step chunk slots of a call that runs in phases.
__constant__ int64_t SEG_PHASE_START[SEG_PHASES + 1] = { 0, 1, 2, 4, 8, 16, 32, 64, INT64_MAX / 4 };
constexpr int64_t SEG_PHASED_MIN_CHUNKS = int64_t(1) << 22;

// Work items [begin, end) and first round of phase p, from the rounds' offsets
// (p < 0: every round in one phase).
__device__ __forceinline__ void phase_items(const int64_t *round_off, int64_t nrounds, int p, int64_t &r0,
                                            int64_t &r1, unsigned long long &begin, unsigned long long &end)
{
	r0 = p < 0 ? 0 : min(SEG_PHASE_START[p], nrounds);
	r1 = p < 0 ? nrounds : min(SEG_PHASE_START[p + 1], nrounds);
	begin = (unsigned long long)round_off[r0];
	end = (unsigned long long)round_off[r1];
}

// Round of work item `item` within rounds [r0, r1): round_off is non-decreasing
// and round_off[r0] <= item < round_off[r1].
__device__ __forceinline__ int64_t round_of(const int64_t *round_off, int64_t r0, int64_t r1, unsigned long long item)
{
	int64_t lo = r0, hi = r1;
	while (hi - lo > 1) {
		const int64_t mid = (lo + hi) >> 1;
		if (round_off[mid] <= (int64_t)item)
			lo = mid;
		else
			hi = mid;
	}
	return lo;
}

// The anchor frames of one round phase: one thread per work item (segment
// chunk, in the traversal's chunk-major order), its anchor step's delta walked
// from the chunk's checkpoint with the reference's update, the FP64 state
// interpolated and reduced to the FP32 frame.  Chunks at or after a contact
// that an earlier phase found are skipped: the traversal skips them as well.
// Kept apart from the traversal so that segments of very different lengths do
// not leave the FP64 lanes of a warp idle.
__global__ void k_seg_anchors(WorldDev W, const double *from, const double *to, const uint32_t *order,
                              const int64_t *round_off, const int64_t *nrounds_p, int phase, const SegParams *params,
                              const double *ckpt, const int32_t *first, QFs *anchors)
{
	int64_t r0, r1;
	unsigned long long begin, end;
	phase_items(round_off, *nrounds_p, phase, r0, r1, begin, end);
	for (unsigned long long item = begin + blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x; item < end;
	     item += (unsigned long long)gridDim.x * blockDim.x) {
		const int64_t j = round_of(round_off, r0, r1, item);
		const uint32_t s = order[item - round_off[j]];
		const SegParams &P = params[s];
		const int64_t K = P.nsteps, k0 = 32 * j;
		if (k0 >= K || (int64_t)first[s] <= k0)
			continue;
		const int cnt = (int)min((int64_t)32, K - k0);
		const double d = pwm::walk_delta(ckpt[P.ckpt_base + j], P.dist, P.step, anchor_of(cnt));
		seg_step_qf(W, from + 7 * (size_t)s, to + 7 * (size_t)s, P, d, anchors[P.ckpt_base + j]);
	}
}

__global__ void k_seg_setup(WorldDev W, const double *from, const double *to, int64_t n, double vdelta, int mode,
                            const int64_t *slots, const int64_t *slot_base, SegParams *params, double *ckpt,
                            int32_t *first, uint32_t *keys, uint32_t *vals, QueryCounters *ctr, int64_t ckpt_cap)
{
	const double rob_r2 = W.rob.r2;
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
	P.inv_stheta = S.linear ? 0.0 : pwm::dvd(1.0, S.stheta);
	P.linear = S.linear;
	P.dist = dist;
	P.inv_dist = pwm::dvd(1.0, dist);
	P.step = step;
	{
		// motion of any robot point per unit tau: |p1 - p0| + (rotation angle 2 theta) * r2;
		// the linear slerp branch turns by less than 1e-7 rad over the whole segment
		const double dx = b[0] - a[0], dy = b[1] - a[1], dz = b[2] - a[2];
		const double lin = sqrt(dx * dx + dy * dy + dz * dz);
		const double ang = S.linear ? 1e-7 : 2.0 * S.theta;
		const double motion = (lin * (1.0 + 1e-12) + ang * rob_r2 * (1.0 + 1e-12)) * (1.0 + 1e-6) + 1e-15;
		P.skip_scale = step * P.inv_dist * (1.0 + 1e-6) * motion + 1e-300;
	}
	P.ckpt_base = slot_base[s];
	int32_t code = INT_MAX;
	int64_t K = 0;
	if (step >= dist || dist != dist) {
		// a NaN distance: the reference loop (delta <= dist) checks no step
		if (dist != dist)
			atomicOr(&ctr->error, (unsigned)PW_DEVERR_NONFINITE);
		code = PW_STEP_NONE;
	} else if (!(step > 0.0) || dist / step > MAX_STEPS) {
		code = -3;
	} else if (P.ckpt_base + slots[s] > ckpt_cap) {
		// graph mode: the reserved checkpoint slots do not hold this segment
		atomicOr(&ctr->error, (unsigned)PW_DEVERR_CKPT_CAP);
		code = -3;
	} else {
		double delta = step;
		const int64_t nslots = slots[s];
		while (delta <= dist) {
			if ((K & 31) == 0) {
				if ((K >> 5) >= nslots) {
					// the step bound was too small: never write past this segment's slots
					atomicOr(&ctr->error, (unsigned)PW_DEVERR_STEP_BOUND);
					code = -3;
					K = 0;
					break;
				}
				ckpt[P.ckpt_base + (K >> 5)] = delta;
				// a chunk that ends well below dist (room counted in FP32, 8 steps of
				// margin) takes every branch of the loop the same way: its 32 updates are
				// taken at once when they stay in one binade, else run as plain adds (same
				// FP64 values, bit for bit)
				const float room = __fdiv_rn((float)pwm::sub(dist, delta), (float)step);
				if (room > 40.f) {
					double r;
					if (pwm::delta_try(delta, dist, step, 32, &r)) {
						delta = r;
					} else {
						for (int i = 0; i < 32; i++)
							delta = pwm::add(delta, step);
					}
					K += 32;
					continue;
				}
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
                                                 int64_t round_cap, int32_t *first, QueryCounters *ctr)
{
	typedef cub::BlockScan<long long, 1024> Scan;
	__shared__ typename Scan::TempStorage tmp;
	__shared__ long long carry;
	int64_t R = n > 0 ? (int64_t)sorted_keys[0] : 0;
	if (R > round_cap) {
		// graph mode: the longest segment has more chunks than reserved; no work runs
		// and every segment reports PW_STEP_INVALID
		for (int64_t i = threadIdx.x; i < n; i += blockDim.x)
			first[i] = PW_STEP_INVALID;
		if (threadIdx.x == 0)
			atomicOr(&ctr->error, (unsigned)PW_DEVERR_ROUND_CAP);
		R = 0;
	}
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
		round_off[round_cap + 1] = R;      // the round count, read by k_segments
		ctr->stat[STAT_TOTAL_ITEMS] = (unsigned long long)carry;
	}
}

// Second pass over a segment chunk some of whose uncertain pairs did not fit the
// FP64 queue: steps 0 .. nopen-1 traversed again with every uncertain pair
// re-tested inline (the anchor frame reloaded first).  Returns the lowest step in
// contact as a one-bit mask.  Not inlined, as resolve_states.
template <bool OBB>
__device__ __noinline__ uint32_t resolve_chunk(const WorldDev &W, WarpSmem &sm, int lane, int nopen, int cnt,
                                               int anchor, float motion, int soft_cap, QueryCounters *ctr,
                                               RetestEntry *rq, const StateSrc &src, LaneStats &st, uint32_t seg,
                                               int64_t ckslot, uint32_t &ndetailed)
{
	if (lane < 5)
		sm.qf[anchor].q[lane] = src.anchors[ckslot].q[lane];
	__syncwarp();
	uint32_t unused = 0;
	return traverse_chunk<RETEST_CAP, true, OBB>(W, sm, lane, nopen, cnt, anchor, motion, soft_cap, ctr, rq, src, st,
	                                        seg, ckslot, ndetailed, unused);
}

// Work item = (segment, 32-step chunk) in chunk-major order, so that early
// contacts prune later chunks; one launch per round phase.  A warp computes the
// chunk's FP64 states lane-parallel, then answers its steps with one swept
// traversal and records the first step in contact with atomicMin.
template <bool OBB>
__global__ void __launch_bounds__(WARPS * 32, 8) k_segments(WorldDev W, StateSrc src, const uint32_t *order,
                                                         const int64_t *round_off, const int64_t *nrounds_p,
                                                         int phase, int32_t *first, QueryCounters *ctr,
                                                         RetestEntry *rq, int soft_cap)
{
	int64_t r0, r1;
	unsigned long long begin, end;
	phase_items(round_off, *nrounds_p, phase, r0, r1, begin, end);
	extern __shared__ __align__(16) unsigned char smem_raw[];
	const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
	WarpSmem &sm = reinterpret_cast<WarpSmem *>(smem_raw)[warp];
	LaneStats st;
	uint32_t queries = 0, items = 0, detailed = 0;
	for (;;) {
		unsigned long long item = 0;
		if (lane == 0)
			item = begin + atomicAdd(&ctr->phase_work[phase < 0 ? 0 : phase], 1ull);
		item = __shfl_sync(FULL, item, 0);
		if (item >= end)
			break;
		int64_t j = 0;
		if (lane == 0)
			j = round_of(round_off, r0, r1, item);
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
		const int anchor = anchor_of(cnt);
		const int64_t ckslot = P.ckpt_base + j;
		if (lane < cnt) {
			sm.slot_query[lane] = s;
			sm.slot_step[lane] = (uint32_t)(k0 + lane);
		}
		if (lane < 5)
			sm.qf[anchor].q[lane] = src.anchors[ckslot].q[lane];
		__syncwarp();
		// steps at or after the segment's current first contact are not needed
		const int lim = (int)min((int64_t)cnt, (int64_t)cur - k0);
		queries += lim;
		const float motion = __double2float_ru(P.skip_scale);
		uint32_t ovf = 0u;
		uint32_t hit = traverse_chunk<RETEST_CAP, false, OBB>(W, sm, lane, lim, cnt, anchor, motion, soft_cap, ctr, rq,
		                                                 src, st, s, ckslot, detailed, ovf);
		// steps below the lowest contact that lost uncertain pairs to a full queue
		if (ovf & (hit ? hit - 1u : FULL)) {
			const uint32_t h2 = resolve_chunk<OBB>(W, sm, lane, hit ? __ffs(hit) - 1 : lim, cnt, anchor, motion,
			                                  soft_cap, ctr, rq, src, st, s, ckslot, detailed);
			if (h2 && (!hit || h2 < hit))
				hit = h2;
		}
		if (hit && lane == 0)
			atomicMin(&first[s], k0 + (__ffs(hit) - 1));
		if (((queries | items) >> 30) || stats_full(st, lane)) {
			flush_stats(ctr, st, queries, items, lane);
			queries = items = 0;
		}
		__syncwarp();
	}
	if (lane == 0 && detailed)
		atomicAdd(&ctr->stat[STAT_DETAILED], (unsigned long long)detailed);
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

// One warp enumerates every leaf pair of the state whose FP32 frame is in
// sm.qf[0] that is not certified separate, calling emit(env face, robot face)
// on the lanes that found one.
template <typename Emit>
__device__ void isect_traverse(const WorldDev &W, WarpSmem &sm, int lane, int soft_cap, Emit emit)
{
	const uint32_t ebase = (uint32_t)W.env.leaf_base, rbase = (uint32_t)W.rob.leaf_base;
	const unsigned gt_mask = ~(((1u << lane) - 1u) | (1u << lane));
	// every contact of a colliding state is enumerated, so there is no early exit to
	// reach sooner: the root pair (seed pairs measured 4 % slower here)
	if (lane == 0)
		sm.stack[0] = make_uint2(0u, 0u);
	__syncwarp();
	const float4 Q0 = sm.qf[0].q[0], Q1 = sm.qf[0].q[1], Q2 = sm.qf[0].q[2], Q3 = sm.qf[0].q[3];
	const float eg = sm.qf[0].q[4].x;
	int top = 1;
	while (top > 0) {
		int p = min(top, 32);
		const int room = soft_cap - top;
		if (room < p)
			p = max(1, room);
		const bool active = lane < p;
		uint2 pr = make_uint2(0u, 0u);
		if (active)
			pr = sm.stack[top - 1 - lane];
		__syncwarp();
		top -= p;
		bool push = false;
		uint2 c0 = make_uint2(0u, 0u), c1 = make_uint2(0u, 0u);
		if (active) {
			const float4 A0 = __ldg(W.env.nodeA + pr.x), A1 = __ldg(W.env.nodeB + pr.x);
			const float4 B0 = __ldg(W.rob.nodeA + pr.y), B1 = __ldg(W.rob.nodeB + pr.y);
			if (!sat_disjoint32(A0, A1, B0, B1, Q0, Q1, Q2, Q3)) {
				const bool la = pr.x >= ebase, lb = pr.y >= rbase;
				if (la && lb) {
					const int es = (int)(pr.x - ebase), rs = (int)(pr.y - rbase);
					const float4 ta = __ldg(W.env.triA + es), tb = __ldg(W.env.triB + es),
					             tc = __ldg(W.env.triC + es);
					const float4 ra = __ldg(W.rob.triA + rs), rb = __ldg(W.rob.triB + rs),
					             rc = __ldg(W.rob.triC + rs);
					float gap;
					const int r = tri_filter(f3(ta), f3(tb), f3(tc), f3(ra), f3(rb), f3(rc), Q0, Q1, Q2, Q3, eg, &gap);
					if (r != 0)
						emit((uint32_t)__float_as_int(ta.w), (uint32_t)__float_as_int(ra.w));
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
			const int o = top + 2 * __popc(pm & gt_mask);
			sm.stack[o] = c1;
			sm.stack[o + 1] = c0;
		}
		top += 2 * __popc(pm);
		__syncwarp();
	}
}

// Candidate pair of a batch: the state and the two original face ids.
struct IsectCand {
	uint32_t state, et, rt, pad;
};

// Persistent warps over a batch of states (one state per warp at a time); the
// candidates of every state go to one buffer of `cap` entries.  *ncand counts
// them all, so a caller sees an overflow as *ncand > cap.
__global__ void __launch_bounds__(WARPS * 32) k_isect_collect_batch(WorldDev W, const double *states, int64_t n,
                                                                    IsectCand *cand, unsigned long long *ncand,
                                                                    unsigned long long cap, unsigned long long *work,
                                                                    int soft_cap)
{
	extern __shared__ __align__(16) unsigned char smem_raw[];
	const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
	WarpSmem &sm = reinterpret_cast<WarpSmem *>(smem_raw)[warp];
	for (;;) {
		unsigned long long i = 0;
		if (lane == 0)
			i = atomicAdd(work, 1ull);
		i = __shfl_sync(FULL, i, 0);
		if (i >= (unsigned long long)n)
			break;
		if (lane == 0) {
			double s[7];
			for (int k = 0; k < 7; k++)
				s[k] = states[7 * i + k];
			make_qf(s, W, sm.qf[0]);
		}
		__syncwarp();
		isect_traverse(W, sm, lane, soft_cap, [&](uint32_t et, uint32_t rt) {
			const unsigned long long idx = atomicAdd(ncand, 1ull);
			if (idx < cap) {
				IsectCand c;
				c.state = (uint32_t)i;
				c.et = et;
				c.rt = rt;
				c.pad = 0;
				cand[idx] = c;
			}
		});
		__syncwarp();
	}
}

struct IsectBatchRow {
	double b[3], e[3], mag;
	int32_t state, et, rt, cop;
};

// FP64 verdict of each candidate of a batch; hits get Moeller's segment at the
// 1e-6 snap, with their state, and count one row of that state.
__global__ void k_isect_eval_batch(WorldDev W, const double *states, const IsectCand *cand,
                                   const unsigned long long *ncand, unsigned long long cap, IsectBatchRow *rows,
                                   unsigned long long *nrows, uint32_t *state_rows)
{
	const unsigned long long cnt = min(*ncand, cap);
	for (unsigned long long i = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x; i < cnt;
	     i += (unsigned long long)gridDim.x * blockDim.x) {
		const IsectCand c = cand[i];
		const double *q = states + 7 * (size_t)c.state;
		double R[9], t[3], U[3][3];
		pwm::state_transform(q, R, t);
		for (int k = 0; k < 3; k++) {
			const int vi = W.rob.F[3 * c.rt + k];
			const double p[3] = { W.rob.V64[3 * vi], W.rob.V64[3 * vi + 1], W.rob.V64[3 * vi + 2] };
			pwm::xform_point(R, t, p, U[k]);
		}
		const double *V0 = W.env.V64 + 3 * W.env.F[3 * c.et + 0];
		const double *V1 = W.env.V64 + 3 * W.env.F[3 * c.et + 1];
		const double *V2 = W.env.V64 + 3 * W.env.F[3 * c.et + 2];
		if (!pwm::tri_tri(V0, V1, V2, U[0], U[1], U[2], 0.0))
			continue;
		IsectBatchRow r;
		int cop = 0;
		pwm::tri_tri_isect(V0, V1, V2, U[0], U[1], U[2], 1e-6, &cop, r.b, r.e);
		const double dx = pwm::sub(r.e[0], r.b[0]), dy = pwm::sub(r.e[1], r.b[1]), dz = pwm::sub(r.e[2], r.b[2]);
		r.mag = pwm::rt(pwm::add(pwm::add(pwm::mul(dx, dx), pwm::mul(dy, dy)), pwm::mul(dz, dz)));
		r.state = (int32_t)c.state;
		r.et = (int32_t)c.et;
		r.rt = (int32_t)c.rt;
		r.cop = cop;
		rows[atomicAdd(nrows, 1ull)] = r;
		atomicAdd(state_rows + c.state, 1u);
	}
}

// Sort keys of the rows: (state, env face, robot face) packed into `bits`
// (state above env above robot face; be + br bits for the faces), or, when
// state_bits is 0, only the two faces.
__global__ void k_isect_keys(const IsectBatchRow *rows, const unsigned long long *nrows, int state_bits, int be,
                             int br, uint64_t *key, uint32_t *idx)
{
	const unsigned long long n = *nrows;
	for (unsigned long long i = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x; i < n;
	     i += (unsigned long long)gridDim.x * blockDim.x) {
		const IsectBatchRow &r = rows[i];
		uint64_t k = ((uint64_t)(uint32_t)r.et << br) | (uint64_t)(uint32_t)r.rt;
		if (state_bits)
			k |= (uint64_t)(uint32_t)r.state << (be + br);
		key[i] = k;
		idx[i] = (uint32_t)i;
	}
}

// The state of each row in the order of a face sort (second pass of a
// two-pass sort when the packed key does not fit 64 bits).
__global__ void k_isect_state_keys(const IsectBatchRow *rows, const unsigned long long *nrows, const uint32_t *idx,
                                   uint32_t *key)
{
	const unsigned long long n = *nrows;
	for (unsigned long long i = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x; i < n;
	     i += (unsigned long long)gridDim.x * blockDim.x)
		key[i] = (uint32_t)rows[idx[i]].state;
}

// Rows in sorted order, split into the caller's arrays.
__global__ void k_isect_gather(const IsectBatchRow *rows, const uint32_t *idx, const unsigned long long *nrows,
                               double *b, double *e, double *mag, int32_t *fp, int32_t *cop)
{
	const unsigned long long n = *nrows;
	for (unsigned long long j = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x; j < n;
	     j += (unsigned long long)gridDim.x * blockDim.x) {
		const IsectBatchRow &r = rows[idx[j]];
		for (int k = 0; k < 3; k++) {
			b[3 * j + k] = r.b[k];
			e[3 * j + k] = r.e[k];
		}
		mag[j] = r.mag;
		fp[2 * j] = r.et;
		fp[2 * j + 1] = r.rt;
		cop[j] = r.cop;
	}
}

// ------------------------------------------------------------------ host helpers

size_t warp_smem_bytes() { return sizeof(WarpSmem); }

int soft_cap_of(const pw_world *w)
{
	const int slack = w->dev.env.depth + w->dev.rob.depth + 5 + 8;   // 5: step-range splits
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
	if (2 * (int64_t)w->dev.rob.ntri - 1 > (int64_t)NODE_MASK)
		return pw_fail(PW_ERR_INVALID_ARG, std::string(who) + ": robot mesh above 2^26 triangles");
	return PW_OK;
}

int ensure_query_scratch(pw_world *w)
{
	PW_CUDA(w->counters.reserve(sizeof(QueryCounters)));
	PW_CUDA(w->retest.reserve(sizeof(RetestEntry) * RETEST_CAP));
	return PW_OK;
}

// Launch configuration of kernel 0 (states) / 1 (segments), as set by pw_world_set_launch_config.
int launch_grid(pw_world *w, int kernel, const void *fn, size_t smem)
{
	const int slot = kernel + 2 * (w->node_boxes[kernel] == PW_BOXES_ORIENTED ? 1 : 0);
	if (w->grid_cache[slot] > 0)
		return w->grid_cache[slot];
	int per_sm = 0;
	cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, WARPS * 32, smem);
	if (per_sm < 1)
		per_sm = 1;
	if (w->launch_blocks[kernel] > 0 && w->launch_blocks[kernel] < per_sm)
		per_sm = w->launch_blocks[kernel];
	w->grid_cache[slot] = per_sm * (w->num_sms > 0 ? w->num_sms : 1);
	return w->grid_cache[slot];
}

int launch_soft_cap(const pw_world *w, int kernel)
{
	const int hard = soft_cap_of(w);
	const int c = w->launch_soft_cap[kernel];
	return c > 0 && c < hard ? c : hard;
}

int launch_width(const pw_world *w, int kernel)
{
	return kernel == 0 && w->launch_width[0] > 0 ? w->launch_width[0] : 32;
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

// The traversal kernels of the world's node-box kind.
template <uint64_t CAP>
const void *states_kernel(const pw_world *w)
{
	return w->node_boxes[0] == PW_BOXES_ORIENTED ? (const void *)k_states<CAP, true>
	                                              : (const void *)k_states<CAP, false>;
}
const void *segments_kernel(const pw_world *w)
{
	return w->node_boxes[1] == PW_BOXES_ORIENTED ? (const void *)k_segments<true> : (const void *)k_segments<false>;
}
template <uint64_t CAP>
void launch_states(const pw_world *w, int grid, size_t smem, cudaStream_t st, const double *states, int64_t n,
                   uint8_t *valid, QueryCounters *ctr, RetestEntry *rq)
{
	if (w->node_boxes[0] == PW_BOXES_ORIENTED)
		k_states<CAP, true><<<grid, WARPS * 32, smem, st>>>(w->dev, states, n, valid, ctr, rq, launch_soft_cap(w, 0),
		                                                    launch_width(w, 0));
	else
		k_states<CAP, false><<<grid, WARPS * 32, smem, st>>>(w->dev, states, n, valid, ctr, rq, launch_soft_cap(w, 0),
		                                                     launch_width(w, 0));
}

} // namespace

// ------------------------------------------------------------------ C ABI

extern "C" int pw_states_valid(pw_world *w, const double *states, int64_t n, uint8_t *valid, void *stream)
{
	PW_TRACE("pw_states_valid");
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
	const void *kfn = states_kernel<RETEST_CAP>(w);
	if (!w->graph_mode && (rc = set_smem_attr(kfn, smem)))
		return rc;
	const int grid = launch_grid(w, 0, kfn, smem);
	RetestEntry *rq = (RetestEntry *)w->retest.ptr;
	if (!w->graph_mode && (rc = mark(w, 0, st)))
		return rc;
	launch_states<RETEST_CAP>(w, grid, smem, st, states, n, valid, ctr, rq);
	w->last_launches = 2;
	if (!w->graph_mode)
		mark(w, 1, st);
	StateSrc src{ states, nullptr, nullptr, nullptr, nullptr, nullptr };
	k_retest<RETEST_CAP><<<w->num_sms * 4, 256, 0, st>>>(w->dev, src, valid, nullptr, ctr, rq);
	if (!w->graph_mode) {
		mark(w, 2, st);
		w->timed = true;
	}
	PW_CUDA(cudaGetLastError());
	return PW_OK;
}

template <typename T>
static int grow(DeviceBuffer &b, size_t count, bool may_allocate = true)
{
	const size_t need = sizeof(T) * (count ? count : 1);
	if (!may_allocate && b.bytes < need)
		return pw_fail(PW_ERR_CAPACITY, "graph mode: scratch not reserved for this batch (call pw_segments_reserve "
		                                "or run the batch once with graph mode off)");
	PW_CUDA(b.reserve(need));
	return PW_OK;
}

extern "C" int pw_states_disentangled(pw_world *w, const double *states, int64_t n, uint8_t *out, void *stream)
{
	PW_TRACE("pw_states_disentangled");
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
	pwm::xform_point(B.Re, B.te, B.ec, B.ce);
	cudaStream_t st = (cudaStream_t)stream;
	int rc = ensure_query_scratch(w);
	if (rc)
		return rc;
	// the queue of undecided states (32-bit state indices, room for all of them)
	if (n > (int64_t)UINT32_MAX)
		return pw_fail(PW_ERR_INVALID_ARG, "pw_states_disentangled: at most 2^32 - 1 states per call");
	if ((rc = grow<uint32_t>(w->dis_queue, (size_t)n)))
		return rc;
	QueryCounters *ctr = (QueryCounters *)w->counters.ptr;
	PW_CUDA(cudaMemsetAsync(ctr, 0, sizeof(QueryCounters), st));
	w->last_stream = st;
	w->timed = false;
	w->last_states = n;
	bool rot = false;
	for (int i = 0; i < 9; i++)
		rot = rot || B.Re[i] != (i % 4 == 0 ? 1.0 : 0.0);
	const void *kfn = rot ? (const void *)k_disentangled<true> : (const void *)k_disentangled<false>;
	int &per_sm = w->dis_per_sm[rot ? 1 : 0];
	if (per_sm <= 0) {
		PW_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kfn, DIS_THREADS, DIS_SMEM));
		per_sm = std::max(per_sm, 1);
	}
	const int64_t blocks = std::min<int64_t>((n + DIS_BLOCK - 1) / DIS_BLOCK, (int64_t)w->num_sms * per_sm);
	uint32_t *queue = (uint32_t *)w->dis_queue.ptr;
	const unsigned grid64 = (unsigned)(w->num_sms * 32);
	if (rot) {
		k_disentangled<true><<<(unsigned)blocks, DIS_THREADS, DIS_SMEM, st>>>(dis_boxes32(B), states, n, out, queue,
		                                                                      ctr);
		k_disentangled64<true><<<grid64, DIS64_BLOCK, 0, st>>>(B, states, queue, n, ctr, out);
	} else {
		k_disentangled<false><<<(unsigned)blocks, DIS_THREADS, DIS_SMEM, st>>>(dis_boxes32(B), states, n, out, queue,
		                                                                       ctr);
		k_disentangled64<false><<<grid64, DIS64_BLOCK, 0, st>>>(B, states, queue, n, ctr, out);
	}
	w->last_launches = 2;
	PW_CUDA(cudaGetLastError());
	return PW_OK;
}


extern "C" int pw_segments_first_contact(pw_world *w, const double *from, const double *to, int64_t n,
                                         double verify_delta, int mode, int32_t *first_step, void *stream)
{
	PW_TRACE("pw_segments_first_contact");
	int rc = check_ready(w, "pw_segments_first_contact");
	if (rc)
		return rc;
	if (n < 0 || (n > 0 && (!from || !to || !first_step)))
		return pw_fail(PW_ERR_INVALID_ARG, "pw_segments_first_contact: bad pointers or size");
	if (mode != PW_SEG_TRANSIT && mode != PW_SEG_TRANSITION)
		return pw_fail(PW_ERR_INVALID_ARG, "pw_segments_first_contact: unknown mode");
	if (2 * (int64_t)w->dev.rob.ntri - 1 > (int64_t)RNODE_MASK)
		return pw_fail(PW_ERR_INVALID_ARG, "pw_segments_first_contact: robot mesh above 2^21 triangles");
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
	w->last_seg_n = -1;
	PW_CUDA(cudaMemsetAsync(ctr, 0, sizeof(QueryCounters), st));
	if (n == 0)
		return PW_OK;
	// scratch: params, slot bounds/base, keys/vals (x2), cub temp
	const bool alloc = !w->graph_mode;
	if ((rc = grow<SegParams>(w->seg_params, n, alloc)) || (rc = grow<int64_t>(w->misc, 2 * n + 2, alloc)) ||
	    (rc = grow<uint32_t>(w->seg_keys, n, alloc)) || (rc = grow<uint32_t>(w->seg_order, n, alloc)) ||
	    (rc = grow<uint32_t>(w->seg_keys2, n, alloc)) || (rc = grow<uint32_t>(w->seg_order2, n, alloc)))
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
	if ((rc = grow<char>(w->cub_tmp, std::max(t1, t2), alloc)))
		return rc;
	// slots[n] = 0 so that slot_base[n] is the total
	PW_CUDA(cudaMemsetAsync(slots + n, 0, sizeof(int64_t), st));
	PW_CUDA(cub::DeviceScan::ExclusiveSum(w->cub_tmp.ptr, t1, slots, slot_base, (int)(n + 1), st));
	int64_t total_slots = -1;   // this call's chunk slots (outside graph mode)
	if (!w->graph_mode) {
		// size the checkpoint arrays by the total (one small synchronous copy)
		PW_CUDA(cudaMemcpyAsync(&total_slots, slot_base + n, sizeof(int64_t), cudaMemcpyDeviceToHost, st));
		PW_CUDA(cudaStreamSynchronize(st));
		if ((rc = grow<double>(w->seg_ckpt, (size_t)total_slots + 1)) ||
		    (rc = grow<QFs>(w->seg_anchor, (size_t)total_slots + 1)))
			return rc;
	}
	const int64_t ckpt_cap = (int64_t)std::min(w->seg_ckpt.bytes / sizeof(double), w->seg_anchor.bytes / sizeof(QFs));
	QFs *anchors = (QFs *)w->seg_anchor.ptr;
	SegParams *params = (SegParams *)w->seg_params.ptr;
	double *ckpt = (double *)w->seg_ckpt.ptr;
	uint32_t *keys = (uint32_t *)w->seg_keys.ptr, *vals = (uint32_t *)w->seg_order.ptr;
	uint32_t *keys2 = (uint32_t *)w->seg_keys2.ptr, *vals2 = (uint32_t *)w->seg_order2.ptr;
	k_seg_setup<<<G, B, 0, st>>>(w->dev, from, to, n, verify_delta, mode, slots, slot_base, params, ckpt,
	                             first_step, keys, vals, ctr, ckpt_cap);
	PW_CUDA(cudaGetLastError());
	PW_CUDA(cub::DeviceRadixSort::SortPairsDescending(w->cub_tmp.ptr, t2, keys, keys2, vals, vals2, (int)n, 0, 32, st));
	if (!w->graph_mode) {
		// rounds: as many as the longest segment has chunks
		uint32_t max_chunks = 0;
		PW_CUDA(cudaMemcpyAsync(&max_chunks, keys2, sizeof(uint32_t), cudaMemcpyDeviceToHost, st));
		PW_CUDA(cudaStreamSynchronize(st));
		if ((int64_t)max_chunks + 2 > (int64_t)(w->round_off.bytes / sizeof(int64_t)) &&
		    (rc = grow<int64_t>(w->round_off, (size_t)max_chunks + 2)))
			return rc;
	}
	if (w->round_off.bytes < 3 * sizeof(int64_t))
		return pw_fail(PW_ERR_CAPACITY, "graph mode: scratch not reserved for this batch");
	const int64_t round_cap = (int64_t)(w->round_off.bytes / sizeof(int64_t)) - 2;
	int64_t *round_off = (int64_t *)w->round_off.ptr;
	k_rounds<<<1, 1024, 0, st>>>(keys2, n, round_off, round_cap, first_step, ctr);
	PW_CUDA(cudaGetLastError());
	const size_t smem = warp_smem_bytes() * WARPS;
	const void *kfn = segments_kernel(w);
	if (!w->graph_mode && (rc = set_smem_attr(kfn, smem)))
		return rc;
	const int grid = launch_grid(w, 1, kfn, smem);
	RetestEntry *rq = (RetestEntry *)w->retest.ptr;
	StateSrc src{ nullptr, from, to, params, ckpt, anchors };
	if (!w->graph_mode && (rc = mark(w, 0, st)))
		return rc;
	// per round phase: the anchor frames of the chunks still needed, then their traversal.
	// Phases pay where there is enough work per phase to keep every warp busy; a
	// smaller batch runs all rounds as one phase (each phase ends with a tail of
	// its slowest chunks).
	const int64_t *nrounds = round_off + round_cap + 1;
	const unsigned agrid = (unsigned)(w->num_sms * 8);
	const int64_t chunk_slots = w->graph_mode ? ckpt_cap : total_slots;
	const bool phased = w->seg_phases == PW_PHASES_ON ||
	                    (w->seg_phases == PW_PHASES_AUTO && chunk_slots >= SEG_PHASED_MIN_CHUNKS);
	for (int p = phased ? 0 : -1; p < (phased ? SEG_PHASES : 0); p++) {
		k_seg_anchors<<<agrid, 256, 0, st>>>(w->dev, from, to, vals2, round_off, nrounds, p, params, ckpt, first_step,
		                                     anchors);
		if (w->node_boxes[1] == PW_BOXES_ORIENTED)
			k_segments<true><<<grid, WARPS * 32, smem, st>>>(w->dev, src, vals2, round_off, nrounds, p, first_step,
			                                                 ctr, rq, launch_soft_cap(w, 1));
		else
			k_segments<false><<<grid, WARPS * 32, smem, st>>>(w->dev, src, vals2, round_off, nrounds, p, first_step,
			                                                  ctr, rq, launch_soft_cap(w, 1));
	}
	PW_CUDA(cudaGetLastError());
	if (!w->graph_mode)
		mark(w, 1, st);
	k_retest<RETEST_CAP><<<w->num_sms * 4, 256, 0, st>>>(w->dev, src, nullptr, first_step, ctr, rq);
	if (!w->graph_mode) {
		mark(w, 2, st);
		w->timed = true;
	}
	k_seg_finalize<<<G, B, 0, st>>>(first_step, params, n, ctr);
	PW_CUDA(cudaGetLastError());
	w->last_launches = 3 + 2 * (phased ? SEG_PHASES : 1) + 2;   // bound, set-up, rounds; the phases; re-test, finalise
	w->last_seg_from = from;
	w->last_seg_to = to;
	w->last_seg_n = n;
	w->last_seg_delta = verify_delta;
	w->last_seg_mode = mode;
	return PW_OK;
}

// Transit tuples from the set-up kernel's checkpoints (the same batch as the
// last pw_segments_first_contact(PW_SEG_TRANSIT) call): at most 31 delta updates
// per state instead of the whole loop up to the first contact.
__global__ void k_contact_states_ckpt(const double *from, const double *to, const SegParams *params,
                                      const double *ckpt, const int32_t *first, int64_t n, double *last_free,
                                      double *contact, uint8_t *done, float *last_tau, float *tau, int *err)
{
	const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
	if (i >= n)
		return;
	const double *a = from + 7 * i, *b = to + 7 * i;
	double *lf = last_free + 7 * i, *st = contact + 7 * i;
	const SegParams &P = params[i];
	const int32_t k = first[i];
	auto state_at = [&](int64_t j, double *q) {
		const double d = pwm::walk_delta(ckpt[P.ckpt_base + (j >> 5)], P.dist, P.step, (int)(j & 31));
		const double t = pwm::mul(d, P.inv_dist);
		pwm::SlerpParams S;
		seg_slerp(P, S);
		pwm::interpolate_p(a, b, S, t, q);
		return t;
	};
	if (k == PW_STEP_NONE) {
		const bool nan = P.dist != P.dist;
		for (int c = 0; c < 7; c++) {
			lf[c] = a[c];
			st[c] = nan ? a[c] : b[c];
		}
		done[i] = 0;
		last_tau[i] = 0.f;
		tau[i] = nan ? 0.f : 1.f;
		return;
	}
	if (k < PW_STEP_NONE || (k == PW_STEP_FREE && P.nsteps <= 0)) {
		atomicCAS(err, 0, 1);
		for (int c = 0; c < 7; c++)
			lf[c] = st[c] = a[c];
		done[i] = 0;
		last_tau[i] = tau[i] = 0.f;
		return;
	}
	if (k >= 0) {
		tau[i] = (float)state_at(k, st);
		if (k == 0) {
			for (int c = 0; c < 7; c++)
				lf[c] = a[c];
			last_tau[i] = 0.f;
		} else {
			last_tau[i] = (float)state_at(k - 1, lf);
		}
		done[i] = 0;
		return;
	}
	const float lt = (float)state_at(P.nsteps - 1, lf);
	for (int c = 0; c < 7; c++)
		st[c] = lf[c];
	done[i] = 1;
	last_tau[i] = lt;
	tau[i] = 0.f;
}

extern "C" int pw_segments_contact_states(const double *from, const double *to, const int32_t *first_step, int64_t n,
                                          double verify_delta, double *last_free, double *contact, uint8_t *done,
                                          float *last_tau, float *tau, int *err_flag, void *stream);

extern "C" int pw_world_segments_contact_states(pw_world *w, const double *from, const double *to,
                                                const int32_t *first_step, int64_t n, double verify_delta,
                                                double *last_free, double *contact, uint8_t *done, float *last_tau,
                                                float *tau, int *err_flag, void *stream)
{
	PW_TRACE("pw_world_segments_contact_states");
	if (!w)
		return pw_fail(PW_ERR_INVALID_ARG, "pw_world_segments_contact_states: world is NULL");
	const bool same = w->last_seg_n == n && w->last_seg_from == from && w->last_seg_to == to &&
	                  w->last_seg_delta == verify_delta && w->last_seg_mode == PW_SEG_TRANSIT &&
	                  w->seg_params.ptr && n > 0;
	w->last_launches += 1;   // either path launches one kernel
	if (!same)
		return pw_segments_contact_states(from, to, first_step, n, verify_delta, last_free, contact, done, last_tau,
		                                  tau, err_flag, stream);
	if (!last_free || !contact || !done || !last_tau || !tau || !err_flag || !first_step)
		return pw_fail(PW_ERR_INVALID_ARG, "pw_world_segments_contact_states: bad pointers");
	PW_CUDA(cudaSetDevice(w->device));
	k_contact_states_ckpt<<<(unsigned)((n + 127) / 128), 128, 0, (cudaStream_t)stream>>>(
	    from, to, (const SegParams *)w->seg_params.ptr, (const double *)w->seg_ckpt.ptr, first_step, n, last_free,
	    contact, done, last_tau, tau, err_flag);
	PW_CUDA(cudaGetLastError());
	return PW_OK;
}

extern "C" int pw_world_set_graph_mode(pw_world *w, int on)
{
	if (!w)
		return pw_fail(PW_ERR_INVALID_ARG, "pw_world_set_graph_mode: world is NULL");
	if (on && w->ready) {
		// the attributes and occupancy queries the launches need, outside any capture
		PW_CUDA(cudaSetDevice(w->device));
		int rc = ensure_query_scratch(w);
		if (rc || (rc = set_smem_attr(segments_kernel(w), warp_smem_bytes() * WARPS)) ||
		    (rc = set_smem_attr(states_kernel<RETEST_CAP>(w), warp_smem_bytes() * WARPS)))
			return rc;
		launch_grid(w, 0, states_kernel<RETEST_CAP>(w), warp_smem_bytes() * WARPS);
		launch_grid(w, 1, segments_kernel(w), warp_smem_bytes() * WARPS);
	}
	w->graph_mode = on != 0;
	return PW_OK;
}

extern "C" int pw_world_scratch_epoch(pw_world *w, uint64_t *out)
{
	if (!w || !out)
		return pw_fail(PW_ERR_INVALID_ARG, "pw_world_scratch_epoch: NULL argument");
	// FNV-1a over the addresses and sizes of every buffer a segment or state query uses
	const DeviceBuffer *bufs[] = { &w->counters, &w->retest, &w->seg_params, &w->seg_ckpt, &w->seg_anchor,
	                               &w->seg_keys, &w->seg_order, &w->seg_keys2, &w->seg_order2, &w->round_off,
	                               &w->cub_tmp, &w->misc };
	uint64_t h = 1469598103934665603ull;
	for (const DeviceBuffer *b : bufs) {
		const uint64_t v[2] = { (uint64_t)(uintptr_t)b->ptr, (uint64_t)b->bytes };
		for (uint64_t x : v)
			for (int i = 0; i < 8; i++) {
				h ^= (x >> (8 * i)) & 0xff;
				h *= 1099511628211ull;
			}
	}
	*out = h;
	return PW_OK;
}

extern "C" int pw_segments_reserve(pw_world *w, int64_t n, int64_t total_chunks, int64_t max_chunks)
{
	PW_TRACE("pw_segments_reserve");
	int rc = check_ready(w, "pw_segments_reserve");
	if (rc)
		return rc;
	if (n < 0 || total_chunks < 0 || max_chunks < 0 || n > (int64_t(1) << 31) - 1)
		return pw_fail(PW_ERR_INVALID_ARG, "pw_segments_reserve: bad sizes");
	PW_CUDA(cudaSetDevice(w->device));
	if ((rc = ensure_query_scratch(w)) || (rc = grow<SegParams>(w->seg_params, n)) ||
	    (rc = grow<int64_t>(w->misc, 2 * n + 2)) || (rc = grow<uint32_t>(w->seg_keys, n)) ||
	    (rc = grow<uint32_t>(w->seg_order, n)) || (rc = grow<uint32_t>(w->seg_keys2, n)) ||
	    (rc = grow<uint32_t>(w->seg_order2, n)) || (rc = grow<double>(w->seg_ckpt, total_chunks + 1)) ||
	    (rc = grow<QFs>(w->seg_anchor, total_chunks + 1)) || (rc = grow<int64_t>(w->round_off, max_chunks + 2)))
		return rc;
	size_t t1 = 0, t2 = 0;
	PW_CUDA(cub::DeviceScan::ExclusiveSum(nullptr, t1, (int64_t *)nullptr, (int64_t *)nullptr, (int)(n + 1)));
	PW_CUDA(cub::DeviceRadixSort::SortPairsDescending(nullptr, t2, (uint32_t *)nullptr, (uint32_t *)nullptr,
	                                                  (uint32_t *)nullptr, (uint32_t *)nullptr, (int)n, 0, 32));
	PW_CUDA(w->cub_tmp.reserve(std::max(t1, t2)));
	return PW_OK;
}

extern "C" int pw_world_set_launch_config(pw_world *w, int kernel, int width, int soft_cap, int blocks)
{
	if (!w || kernel < 0 || kernel > 1 || width < 0 || width > 32 || soft_cap < 0 || blocks < 0)
		return pw_fail(PW_ERR_INVALID_ARG, "pw_world_set_launch_config: bad argument");
	if (soft_cap > 0 && soft_cap < 64)
		return pw_fail(PW_ERR_INVALID_ARG, "pw_world_set_launch_config: soft_cap below 64");
	w->launch_width[kernel] = width;
	w->launch_soft_cap[kernel] = soft_cap;
	w->launch_blocks[kernel] = blocks;
	w->grid_cache[kernel] = w->grid_cache[kernel + 2] = 0;
	return PW_OK;
}

extern "C" int pw_world_get_launch_config(pw_world *w, int kernel, int *width, int *soft_cap, int *blocks)
{
	if (!w || kernel < 0 || kernel > 1 || !width || !soft_cap || !blocks)
		return pw_fail(PW_ERR_INVALID_ARG, "pw_world_get_launch_config: bad argument");
	*width = launch_width(w, kernel);
	*soft_cap = w->ready ? launch_soft_cap(w, kernel) : w->launch_soft_cap[kernel];
	*blocks = w->launch_blocks[kernel];
	if (*blocks == 0 && w->ready) {
		const void *k = kernel == 0 ? states_kernel<RETEST_CAP>(w) : segments_kernel(w);
		PW_CUDA(cudaSetDevice(w->device));
		int rc = set_smem_attr(k, warp_smem_bytes() * WARPS);
		if (rc)
			return rc;
		*blocks = launch_grid(w, kernel, k, warp_smem_bytes() * WARPS) / (w->num_sms > 0 ? w->num_sms : 1);
	}
	return PW_OK;
}

// Candidate pairs one chunk of a contact enumeration holds on the device, and
// the most states of one chunk.  The chunk's state count follows the
// candidates per state seen so far; a chunk whose candidates overflow is
// re-run with fewer states.
constexpr unsigned long long ISECT_BATCH_CAP = 1ull << 22;
constexpr int64_t ISECT_BATCH_CHUNK = 65536;

// The world's contact-enumeration scratch, carved from one buffer.
struct IsectScratch {
	double *q;                 // ISECT_BATCH_CHUNK states
	unsigned long long *ctr;   // candidates, rows, work
	uint32_t *state_rows;      // rows per state of the chunk
	int64_t *row_end;          // inclusive scan of state_rows
	IsectCand *cand;
	IsectBatchRow *rows;
	uint64_t *key[2];
	uint32_t *idx[2];
	double *b, *e, *mag;
	int32_t *fp, *cop;
	void *tmp;
	size_t tmp_bytes;
};

static int isect_scratch(pw_world *w, IsectScratch &S)
{
	const size_t C = ISECT_BATCH_CAP, M = ISECT_BATCH_CHUNK;
	size_t t1 = 0, t2 = 0, t3 = 0;
	PW_CUDA(cub::DeviceRadixSort::SortPairs(nullptr, t1, (uint64_t *)nullptr, (uint64_t *)nullptr,
	                                        (uint32_t *)nullptr, (uint32_t *)nullptr, (int)C, 0, 64));
	PW_CUDA(cub::DeviceRadixSort::SortPairs(nullptr, t2, (uint32_t *)nullptr, (uint32_t *)nullptr,
	                                        (uint32_t *)nullptr, (uint32_t *)nullptr, (int)C, 0, 32));
	PW_CUDA(cub::DeviceScan::InclusiveSum(nullptr, t3, (const uint32_t *)nullptr, (int64_t *)nullptr, (int)M));
	S.tmp_bytes = std::max(t1, std::max(t2, t3));
	const size_t sizes[] = { sizeof(double) * 7 * M, sizeof(unsigned long long) * 4, sizeof(uint32_t) * M,
		                     sizeof(int64_t) * M, sizeof(IsectCand) * C, sizeof(IsectBatchRow) * C,
		                     sizeof(uint64_t) * C, sizeof(uint64_t) * C, sizeof(uint32_t) * C, sizeof(uint32_t) * C,
		                     sizeof(double) * 3 * C, sizeof(double) * 3 * C, sizeof(double) * C,
		                     sizeof(int32_t) * 2 * C, sizeof(int32_t) * C, S.tmp_bytes };
	constexpr int NS = sizeof(sizes) / sizeof(sizes[0]);
	size_t off[NS], total = 0;
	for (int i = 0; i < NS; i++) {
		off[i] = total;
		total += (sizes[i] + 255) & ~(size_t)255;
	}
	PW_CUDA(w->isect.reserve(total));
	uint8_t *p = (uint8_t *)w->isect.ptr;
	S.q = (double *)(p + off[0]);
	S.ctr = (unsigned long long *)(p + off[1]);
	S.state_rows = (uint32_t *)(p + off[2]);
	S.row_end = (int64_t *)(p + off[3]);
	S.cand = (IsectCand *)(p + off[4]);
	S.rows = (IsectBatchRow *)(p + off[5]);
	S.key[0] = (uint64_t *)(p + off[6]);
	S.key[1] = (uint64_t *)(p + off[7]);
	S.idx[0] = (uint32_t *)(p + off[8]);
	S.idx[1] = (uint32_t *)(p + off[9]);
	S.b = (double *)(p + off[10]);
	S.e = (double *)(p + off[11]);
	S.mag = (double *)(p + off[12]);
	S.fp = (int32_t *)(p + off[13]);
	S.cop = (int32_t *)(p + off[14]);
	S.tmp = p + off[15];
	return PW_OK;
}

// Host copies split over threads: a large result's first touch of the
// caller's fresh pages (its page faults) is what these copies cost, and the
// faults of different threads proceed in parallel.
struct HostCopy {
	void *dst;
	const void *src;
	size_t bytes;
};
static void parallel_copy(const std::vector<HostCopy> &jobs)
{
	size_t total = 0;
	for (const HostCopy &j : jobs)
		total += j.bytes;
	const unsigned hw = std::thread::hardware_concurrency();
	const unsigned T = (unsigned)std::max<size_t>(1, std::min<size_t>({ (size_t)(hw ? hw : 1), (size_t)16,
	                                                                    total / (size_t(4) << 20) }));
	if (T <= 1) {
		for (const HostCopy &j : jobs)
			if (j.bytes)
				memcpy(j.dst, j.src, j.bytes);
		return;
	}
	// thread t copies bytes [t * per, (t + 1) * per) of the jobs laid end to end
	const size_t per = (total + T - 1) / T;
	auto work = [&jobs, per](unsigned t) {
		size_t lo = t * per, hi = lo + per, at = 0;
		for (const HostCopy &j : jobs) {
			const size_t a = std::max(lo, at), b = std::min(hi, at + j.bytes);
			if (a < b)
				memcpy((char *)j.dst + (a - at), (const char *)j.src + (a - at), b - a);
			at += j.bytes;
		}
	};
	std::vector<std::thread> th;
	th.reserve(T - 1);
	for (unsigned t = 1; t < T; t++)
		th.emplace_back(work, t);
	work(0);
	for (std::thread &x : th)
		x.join();
}

static int bits_for(int64_t count) // bits of the largest index below count
{
	int b = 1;
	while (b < 63 && (int64_t(1) << b) < count)
		b++;
	return b;
}

// Contact enumeration of n states (host arrays): rows of state i at
// offsets[i] .. offsets[i + 1] - 1, sorted by (env face, robot face); rows past
// `capacity` are not written.  who names the entry point in errors.
static int isect_run(pw_world *w, const double *q, int64_t n, int64_t capacity, double *begins, double *ends,
                     double *mags, int32_t *face_pairs, int32_t *coplanar, int64_t *offsets, int64_t *total,
                     const char *who)
{
	*total = 0;
	for (int64_t i = 0; i <= n; i++)
		offsets[i] = 0;
	if (n == 0 || w->dev.env.ntri == 0 || w->dev.rob.ntri == 0)
		return PW_OK;
	PW_CUDA(cudaSetDevice(w->device));
	IsectScratch S;
	int rc = isect_scratch(w, S);
	if (rc)
		return rc;
	const size_t smem = warp_smem_bytes() * WARPS;
	if ((rc = set_smem_attr((const void *)k_isect_collect_batch, smem)))
		return rc;
	int per_sm = 0;
	PW_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_isect_collect_batch, WARPS * 32, smem));
	const int grid = std::max(1, per_sm) * std::max(1, w->num_sms);
	const int egrid = std::max(1, w->num_sms) * 8;
	const int be = bits_for(w->dev.env.ntri), br = bits_for(w->dev.rob.ntri);
	std::vector<int64_t> ends_h;
	int64_t chunk = std::min<int64_t>(n, ISECT_BATCH_CHUNK), base = 0;
	unsigned long long launches = 0, tested = 0;
	// a chunk's output columns go to one half of the pinned stage; their copy into the
	// caller's arrays runs while the next chunk's candidates are collected
	constexpr size_t ROW_BYTES = 7 * sizeof(double) + 3 * sizeof(int32_t);
	std::vector<HostCopy> pending;
	int half = 0;
	for (int64_t s0 = 0; s0 < n;) {
		const int64_t m = std::min(chunk, n - s0);
		PW_CUDA(cudaMemcpy(S.q, q + 7 * s0, sizeof(double) * 7 * (size_t)m, cudaMemcpyHostToDevice));
		PW_CUDA(cudaMemset(S.ctr, 0, sizeof(unsigned long long) * 3));
		PW_CUDA(cudaMemset(S.state_rows, 0, sizeof(uint32_t) * (size_t)m));
		k_isect_collect_batch<<<grid, WARPS * 32, smem>>>(w->dev, S.q, m, S.cand, S.ctr, ISECT_BATCH_CAP, S.ctr + 2,
		                                                 soft_cap_of(w));
		PW_CUDA(cudaGetLastError());
		launches++;
		parallel_copy(pending);
		pending.clear();
		unsigned long long c[2];
		PW_CUDA(cudaMemcpy(c, S.ctr, sizeof(c), cudaMemcpyDeviceToHost));
		if (c[0] > ISECT_BATCH_CAP) {
			if (m == 1)
				return pw_fail(PW_ERR_CAPACITY, std::string(who) + ": a state has more than 2^22 candidate pairs");
			chunk = std::max<int64_t>(1, std::min<int64_t>(m / 2, (int64_t)((double)m * 0.8 * ISECT_BATCH_CAP / c[0])));
			continue;
		}
		k_isect_eval_batch<<<egrid, 256>>>(w->dev, S.q, S.cand, S.ctr, ISECT_BATCH_CAP, S.rows, S.ctr + 1,
		                                   S.state_rows);
		PW_CUDA(cudaGetLastError());
		launches++;
		tested += c[0];
		PW_CUDA(cudaMemcpy(c, S.ctr, sizeof(c), cudaMemcpyDeviceToHost));
		const int64_t nr = (int64_t)c[1];
		size_t tb = S.tmp_bytes;
		PW_CUDA(cub::DeviceScan::InclusiveSum(S.tmp, tb, (const uint32_t *)S.state_rows, S.row_end, (int)m));
		ends_h.resize((size_t)m);
		PW_CUDA(cudaMemcpy(ends_h.data(), S.row_end, sizeof(int64_t) * (size_t)m, cudaMemcpyDeviceToHost));
		if (ends_h[(size_t)m - 1] != nr)
			return pw_fail(PW_ERR_INTERNAL, std::string(who) + ": row counts disagree");
		for (int64_t i = 0; i < m; i++)
			offsets[s0 + i + 1] = base + ends_h[(size_t)i];
		if (nr > 0 && base + nr <= capacity) {
			const int sb = bits_for(m);
			const uint32_t *order;
			k_isect_keys<<<egrid, 256>>>(S.rows, S.ctr + 1, sb + be + br <= 64 ? sb : 0, be, br, S.key[0],
			                             S.idx[0]);
			PW_CUDA(cudaGetLastError());
			tb = S.tmp_bytes;
			if (sb + be + br <= 64) {
				PW_CUDA(cub::DeviceRadixSort::SortPairs(S.tmp, tb, S.key[0], S.key[1], S.idx[0], S.idx[1], (int)nr, 0,
				                                        sb + be + br));
				order = S.idx[1];
			} else {
				// faces first, then a stable sort by state
				PW_CUDA(cub::DeviceRadixSort::SortPairs(S.tmp, tb, S.key[0], S.key[1], S.idx[0], S.idx[1], (int)nr, 0,
				                                        be + br));
				uint32_t *k32a = (uint32_t *)S.key[0], *k32b = (uint32_t *)S.key[1];
				k_isect_state_keys<<<egrid, 256>>>(S.rows, S.ctr + 1, S.idx[1], k32a);
				PW_CUDA(cudaGetLastError());
				tb = S.tmp_bytes;
				PW_CUDA(cub::DeviceRadixSort::SortPairs(S.tmp, tb, k32a, k32b, S.idx[1], S.idx[0], (int)nr, 0, sb));
				order = S.idx[0];
				launches++;
			}
			k_isect_gather<<<egrid, 256>>>(S.rows, order, S.ctr + 1, S.b, S.e, S.mag, S.fp, S.cop);
			PW_CUDA(cudaGetLastError());
			launches += 2;
			// the columns, back to back in this chunk's half of the stage
			const size_t cb[5] = { sizeof(double) * 3 * (size_t)nr, sizeof(double) * 3 * (size_t)nr,
				                   sizeof(double) * (size_t)nr, sizeof(int32_t) * 2 * (size_t)nr,
				                   sizeof(int32_t) * (size_t)nr };
			const void *from[5] = { S.b, S.e, S.mag, S.fp, S.cop };
			void *to[5] = { begins + 3 * base, ends + 3 * base, mags + base, face_pairs + 2 * base,
				            coplanar ? (void *)(coplanar + base) : nullptr };
			const size_t need = ROW_BYTES * (size_t)nr;
			if (w->isect_stage.bytes < 2 * need) {
				// a larger stage: the copies still pending read the old one
				parallel_copy(pending);
				pending.clear();
				PW_CUDA(w->isect_stage.reserve(2 * (need + need / 4)));
			}
			const size_t half_bytes = w->isect_stage.bytes / 2;
			char *stage = (char *)w->isect_stage.ptr + half * half_bytes;
			size_t at = 0;
			for (int k = 0; k < 5; k++) {
				if (!to[k])
					continue;
				PW_CUDA(cudaMemcpyAsync(stage + at, from[k], cb[k], cudaMemcpyDeviceToHost, 0));
				pending.push_back(HostCopy{ to[k], stage + at, cb[k] });
				at += cb[k];
			}
			PW_CUDA(cudaStreamSynchronize(0));
			half ^= 1;
		}
		base += nr;
		s0 += m;
		if (c[0] > 0)
			chunk = std::max<int64_t>(1, std::min<int64_t>(ISECT_BATCH_CHUNK,
			                                               (int64_t)((double)m * 0.8 * ISECT_BATCH_CAP / c[0])));
		else
			chunk = ISECT_BATCH_CHUNK;
	}
	parallel_copy(pending);
	*total = base;
	// the figures pw_world_last_stats reports for this query
	if ((rc = ensure_query_scratch(w)))
		return rc;
	QueryCounters hc;
	memset(&hc, 0, sizeof(hc));
	hc.stat[STAT_QUERIES] = (unsigned long long)n;
	hc.stat[STAT_RETESTS] = tested;
	hc.stat[STAT_RETEST_HITS] = (unsigned long long)base;
	hc.stat[STAT_ITEMS] = launches;
	PW_CUDA(cudaMemcpy(w->counters.ptr, &hc, sizeof(hc), cudaMemcpyHostToDevice));
	w->last_states = n;
	w->last_stream = nullptr;
	w->timed = false;
	w->last_launches = (int64_t)launches;
	if (capacity < base)
		return pw_fail(PW_ERR_CAPACITY, std::string(who) + ": capacity smaller than the row count");
	return PW_OK;
}

extern "C" int pw_intersecting_segments(pw_world *w, const double q[7], int64_t capacity, double *begins,
                                        double *ends, double *mags, int32_t *face_pairs, int32_t *coplanar,
                                        int64_t *count)
{
	PW_TRACE("pw_intersecting_segments");
	int rc = check_ready(w, "pw_intersecting_segments");
	if (rc)
		return rc;
	if (!q || !count || capacity < 0 || (capacity > 0 && (!begins || !ends || !mags || !face_pairs)))
		return pw_fail(PW_ERR_INVALID_ARG, "pw_intersecting_segments: bad argument");
	int64_t offsets[2];
	return isect_run(w, q, 1, capacity, begins, ends, mags, face_pairs, coplanar, offsets, count,
	                 "pw_intersecting_segments");
}

extern "C" int pw_intersecting_segments_batch(pw_world *w, const double *q, int64_t n, int64_t capacity,
                                              double *begins, double *ends, double *mags, int32_t *face_pairs,
                                              int32_t *coplanar, int64_t *offsets, int64_t *total)
{
	PW_TRACE("pw_intersecting_segments_batch");
	int rc = check_ready(w, "pw_intersecting_segments_batch");
	if (rc)
		return rc;
	if (n < 0 || capacity < 0 || !offsets || !total || (n > 0 && !q) ||
	    (capacity > 0 && (!begins || !ends || !mags || !face_pairs)))
		return pw_fail(PW_ERR_INVALID_ARG, "pw_intersecting_segments_batch: bad pointers or sizes");
	if (n > (int64_t(1) << 31))
		return pw_fail(PW_ERR_INVALID_ARG, "pw_intersecting_segments_batch: at most 2^31 states per call");
	return isect_run(w, q, n, capacity, begins, ends, mags, face_pairs, coplanar, offsets, total,
	                 "pw_intersecting_segments_batch");
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
	out->detailed_chunks = (int64_t)c.stat[STAT_DETAILED];
	out->device_errors = (int64_t)c.error;
	out->kernel_launches = w->last_launches;
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
	PW_TRACE("pw_states_valid_noalloc");
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
	rc = set_smem_attr(states_kernel<NOALLOC_RETEST_CAP>(w), smem);
	if (rc)
		return rc;
	// the world's launch configuration, as pw_states_valid uses it (both instances of the
	// kernel have the same resources, so they share the cached grid)
	const int grid = launch_grid(w, 0, states_kernel<NOALLOC_RETEST_CAP>(w), smem);
	launch_states<NOALLOC_RETEST_CAP>(w, grid, smem, st, states, n, valid, ctr, rq);
	w->last_launches = 2;
	StateSrc src{ states, nullptr, nullptr, nullptr, nullptr, nullptr };
	k_retest<NOALLOC_RETEST_CAP><<<w->num_sms * 4, 256, 0, st>>>(w->dev, src, valid, nullptr, ctr, rq);
	PW_CUDA(cudaGetLastError());
	return PW_OK;
}

extern "C" int pw_world_set_node_boxes(pw_world *w, int kernel, int kind)
{
	if (!w || kernel < -1 || kernel > 1 || (kind != PW_BOXES_ALIGNED && kind != PW_BOXES_ORIENTED))
		return pw_fail(PW_ERR_INVALID_ARG, "pw_world_set_node_boxes: bad argument");
	if (w->graph_mode)
		return pw_fail(PW_ERR_INVALID_ARG, "pw_world_set_node_boxes: not in graph mode (captured launches hold the kernel)");
	for (int k = 0; k < 2; k++)
		if (kernel < 0 || kernel == k)
			w->node_boxes[k] = kind;
	return PW_OK;
}

extern "C" int pw_world_get_node_boxes(pw_world *w, int kernel, int *kind)
{
	if (!w || !kind || kernel < 0 || kernel > 1)
		return pw_fail(PW_ERR_INVALID_ARG, "pw_world_get_node_boxes: bad argument");
	*kind = w->node_boxes[kernel];
	return PW_OK;
}

extern "C" int pw_world_set_segment_phases(pw_world *w, int mode)
{
	if (!w || (mode != PW_PHASES_AUTO && mode != PW_PHASES_OFF && mode != PW_PHASES_ON))
		return pw_fail(PW_ERR_INVALID_ARG, "pw_world_set_segment_phases: bad argument");
	if (w->graph_mode)
		return pw_fail(PW_ERR_INVALID_ARG,
		               "pw_world_set_segment_phases: not in graph mode (captured launches hold the phases)");
	w->seg_phases = mode;
	return PW_OK;
}

extern "C" int pw_world_get_segment_phases(pw_world *w, int *mode)
{
	if (!w || !mode)
		return pw_fail(PW_ERR_INVALID_ARG, "pw_world_get_segment_phases: bad argument");
	*mode = w->seg_phases;
	return PW_OK;
}
