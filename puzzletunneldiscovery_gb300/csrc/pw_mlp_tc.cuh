// pw_mlp_tc.cuh -- fused forward pass of the proposal network on the 5th-generation
// tensor cores (tcgen05 + tensor memory), sm_103a.  Included by pw_mlp.cu inside
// its anonymous namespace (uses H, KIN, bf16, tanh_fast, feature_row).
//
// One persistent CTA per SM walks pairs of 128-row tiles of states (slots A
// and B).  Each slot owns one 64 KB activation buffer (shared memory, BF16,
// 128-byte swizzle) and one 256-column FP32 accumulator in tensor memory.
// Per slot and layer l:
//   MMA thread: act x W_l^T -> acc (K-blocks of 64, streamed weight blocks)
//   epilogue warps: acc + b_l -> SiLU -> act (BF16), for layers 1..3;
//                   layer 4: SiLU, dot with w5, + b5 -> logit or sigmoid
// The MMA thread issues A(l), B(l), A(l+1), B(l+1), ... so the epilogue of one
// slot runs while the tensor cores work on the other.
// Weights are stored pre-scaled by 1/2 (exact in BF16 and FP32), so the
// accumulator holds h = z / 2 and SiLU(z) = h + h tanh(h) costs one FADD (bias),
// one MUFU and one FFMA per element.
// Weights stream through a 3-stage ring of 32 KB blocks (256 rows x 64 k), each
// one bulk copy of an image already in the swizzled layout the MMA reads
// (built by k_weight_image).  The ring is used as a cache: slot B takes each
// layer's K-blocks in reverse order, so three of the four blocks slot A used
// are still resident (a pair loads 16 blocks instead of 26; schedule below).
//
// Roles (576 threads): warp 0 = weight producer and TMEM owner, warp 1 = MMA
// issuer, warps 2..17 = epilogue (warp w reads TMEM lanes 32 (w % 4) ..).
// Every wait is an mbarrier try_wait bounded by a wall-clock limit; on
// expiry the kernel records an error, stops all roles, waits (bounded) for
// its copies and MMAs in flight, frees its tensor memory and returns.

namespace tc {

constexpr int TILE_M = 128;
constexpr int KB = 64;                        // k per weight block / act K-block
constexpr int NSTAGE = 3;
constexpr int WBLOCK_BYTES = H * KB * 2;      // 32 KB: 256 rows x 128 bytes
constexpr int NWBLOCK = 1 + 3 * (H / KB);     // W1 (one block) + 4 blocks for each of W2..W4
constexpr int ACT_KB_BYTES = TILE_M * KB * 2; // 16 KB per act K-block
constexpr int ACT_BYTES = 4 * ACT_KB_BYTES;   // 64 KB per slot
constexpr int NEPI_WARPS = 16;
constexpr int NTHREADS = (2 + NEPI_WARPS) * 32;
constexpr uint64_t WAIT_LIMIT_NS = 2000000000ull;   // 2 s per wait

// shared-memory map (offsets from a 1024-byte aligned base)
constexpr int SM_ACT = 0;                                        // 2 slots x 64 KB
constexpr int SM_W = SM_ACT + 2 * ACT_BYTES;                     // NSTAGE x 32 KB
constexpr int SM_BAR = SM_W + NSTAGE * WBLOCK_BYTES;             // mbarriers
constexpr int NBAR = 2 * NSTAGE + 2 + 2 + 2 + 1;                 // full, empty, act, done, head, final
constexpr int SM_MISC = SM_BAR + NBAR * 8;                       // tmem base, abort flag
constexpr int SMEM_BYTES = SM_MISC + 16 + 1024;                  // + alignment slack
static_assert(SMEM_BYTES <= 232448, "shared memory budget of one CTA");

// barrier indices (act, done, head: one per slot)
constexpr int B_FULL = 0, B_EMPTY = NSTAGE, B_ACT = 2 * NSTAGE, B_DONE = B_ACT + 2, B_HEAD = B_DONE + 2,
              B_FINAL = B_HEAD + 2;

using pwa::bulk_g2s;
using pwa::mbar_arrive;
using pwa::mbar_expect_tx;
using pwa::mbar_init;
using pwa::mbar_test;
using pwa::now_ns;
using pwa::smem_u32;

// Waits for the phase of `parity` to complete.  Gives up when another role has
// aborted or after WAIT_LIMIT_NS, recording `where` in *err; returns false then.
__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t parity, volatile int *abort_flag, int *err, int where)
{
	if (mbar_test(bar, parity))
		return true;
	const uint64_t t0 = now_ns();
	for (;;) {
		if (mbar_test(bar, parity))
			return true;
		if (*abort_flag)
			return false;
		if (now_ns() - t0 > WAIT_LIMIT_NS) {
			*abort_flag = 1;
			atomicCAS(err, 0, where);
			return false;
		}
	}
}

// Waits for a phase without watching the abort flag (teardown: copies and MMAs in flight).
__device__ __forceinline__ void mbar_drain(uint32_t bar, uint32_t parity)
{
	const uint64_t t0 = now_ns();
	while (!mbar_test(bar, parity) && now_ns() - t0 < WAIT_LIMIT_NS) {
	}
}

// Shared-memory matrix descriptor: K-major operand, 128-byte swizzle, rows of
// 128 bytes, 8-row groups 1024 bytes apart (SBO), descriptor version 1.
__device__ __forceinline__ uint64_t sdesc(uint32_t addr)
{
	return (uint64_t)((addr >> 4) & 0x3FFF) | ((uint64_t)1 << 16) | ((uint64_t)(1024 >> 4) << 32) |
	       ((uint64_t)1 << 46) | ((uint64_t)2 << 61);
}

// Instruction descriptor, kind::f16: D F32, A and B BF16, both K-major, M = 128, N = 256.
constexpr uint32_t IDESC = (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(256 >> 3) << 17) |
                           ((uint32_t)(128 >> 4) << 24);

__device__ __forceinline__ void mma_bf16_ss(uint32_t d_tmem, uint64_t a, uint64_t b, uint32_t accumulate)
{
	asm volatile("{\n\t.reg .pred p;\n\t"
	             "setp.ne.b32 p, %4, 0;\n\t"
	             "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(d_tmem),
	             "l"(a), "l"(b), "r"(IDESC), "r"(accumulate)
	             : "memory");
}
__device__ __forceinline__ void mma_commit(uint32_t bar)
{
	asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(bar)
	             : "memory");
}
__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void fence_async_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

__device__ __forceinline__ void tmem_ld16_nw(uint32_t taddr, uint32_t r[16])
{
	asm volatile("tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, "
	             "[%16];"
	             : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
	               "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]),
	               "=r"(r[15])
	             : "r"(taddr));
}
__device__ __forceinline__ void tmem_wait_ld() { asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory"); }

__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float v[16])
{
	uint32_t r[16];
	asm volatile("tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, "
	             "[%16];"
	             : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
	               "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]),
	               "=r"(r[15])
	             : "r"(taddr));
	asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
	for (int i = 0; i < 16; i++)
		v[i] = __uint_as_float(r[i]);
}

// Byte offset of the 16-byte chunk `c` (0..7) of row `r` in a 128-byte-swizzled K-block.
__device__ __forceinline__ uint32_t swz(int r, int c) { return (uint32_t)(r * 128 + ((c ^ (r & 7)) << 4)); }

__device__ __forceinline__ uint32_t pack_bf16x2(float a, float b)
{
	__nv_bfloat162 h = __floats2bfloat162_rn(a, b);
	return *reinterpret_cast<uint32_t *>(&h);
}

// SiLU of two pre-activations (accumulator + bias, both halved by the weight
// scaling), packed to BF16: with h = x / 2, SiLU(x) = h + h tanh(h).  The add and
// the fma run as packed f32x2 instructions (two lanes per instruction, each
// rounded as its scalar form).
__device__ __forceinline__ uint32_t silu_pair(uint32_t acc0, uint32_t acc1, float b0, float b1)
{
	uint64_t h, b, t, y;
	asm("mov.b64 %0, {%1, %2};" : "=l"(h) : "r"(acc0), "r"(acc1));
	asm("mov.b64 %0, {%1, %2};" : "=l"(b) : "f"(b0), "f"(b1));
	asm("add.rn.f32x2 %0, %1, %2;" : "=l"(h) : "l"(h), "l"(b));
	float h0, h1;
	asm("mov.b64 {%0, %1}, %2;" : "=f"(h0), "=f"(h1) : "l"(h));
	const float t0 = tanh_fast(h0), t1 = tanh_fast(h1);
	asm("mov.b64 %0, {%1, %2};" : "=l"(t) : "f"(t0), "f"(t1));
	asm("fma.rn.f32x2 %0, %1, %2, %1;" : "=l"(y) : "l"(h), "l"(t));
	float y0, y1;
	asm("mov.b64 {%0, %1}, %2;" : "=f"(y0), "=f"(y1) : "l"(y));
	return pack_bf16x2(y0, y1);
}

// Per-column constants of the epilogue, after the weight images:
// [4][256] biases b_l / 2, [256] w5, b5 (16-byte aligned rows).
constexpr int HT_W5 = 4 * H, HT_B5 = 5 * H, HT_FLOATS = 5 * H + 4;

// Weight-block schedule of one pair of tiles (entry i = i-th use of a block by
// the MMA thread), built on the host by pw_mlp.cu: slot B walks the K-blocks of
// each layer in reverse, so the blocks slot A left in the ring are used again
// without a reload.  Entry bits: 0-3 block, 4-5 stage, 6 load before use,
// 7 last use of the stage's content (release it), 8-9 K-block j of the act.
constexpr int SCHED_MAX = 2 + 3 * 8;
struct Sched {
	int n[2];                          // uses of a pair with 1 / 2 live slots
	uint16_t e[2][SCHED_MAX];
};
__device__ __forceinline__ int se_block(uint16_t e) { return e & 15; }
__device__ __forceinline__ int se_stage(uint16_t e) { return (e >> 4) & 3; }
__device__ __forceinline__ bool se_load(uint16_t e) { return (e >> 6) & 1; }
__device__ __forceinline__ bool se_last(uint16_t e) { return (e >> 7) & 1; }
__device__ __forceinline__ int se_kb(uint16_t e) { return (e >> 8) & 3; }

struct FwdArgs {
	Sched sched;
	const double *states;
	int64_t n;
	const bf16 *wimg;        // NWBLOCK images of WBLOCK_BYTES (weights scaled by 1/2)
	float *prob;
	int logits;              // 1: write the logit (a ranking score that does not saturate) instead of P(free)
	int withhold;            // 1: issue no weight copies (the test of the bounded waits: they run out)
	int *err;
	float ht[HT_FLOATS];     // epilogue constants (HT_*), in the launch's parameter bank
};

__global__ void __launch_bounds__(NTHREADS, 1) k_mlp_forward_tc(FwdArgs a)
{
	extern __shared__ uint8_t smem_raw[];
	uint8_t *sm = (uint8_t *)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
	const uint32_t sbase = smem_u32(sm);
	uint32_t *s_tmem = (uint32_t *)(sm + SM_MISC);
	volatile int *s_abort = (volatile int *)(sm + SM_MISC + 4);
	auto bar = [&](int i) { return sbase + SM_BAR + 8 * i; };

	const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
	const int64_t ntiles = (a.n + TILE_M - 1) / TILE_M;
	const int64_t G = gridDim.x;

	if (threadIdx.x == 0) {
		for (int s = 0; s < NSTAGE; s++) {
			mbar_init(bar(B_FULL + s), 1);
			mbar_init(bar(B_EMPTY + s), 1);
		}
		for (int sl = 0; sl < 2; sl++) {
			mbar_init(bar(B_ACT + sl), NEPI_WARPS);
			mbar_init(bar(B_DONE + sl), 1);
			mbar_init(bar(B_HEAD + sl), NEPI_WARPS);
		}
		mbar_init(bar(B_FINAL), 1);
		*s_abort = 0;
		asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
	}
	if (warp == 0) {
		asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], 512;" ::"r"(smem_u32(s_tmem))
		             : "memory");
		asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
	}
	tc_fence_before();
	__syncthreads();
	tc_fence_after();
	const uint32_t tmem = *s_tmem;

	if (warp == 0) {
		// ---------------- weight producer: the loads of the pair's schedule, in order
		if (lane == 0) {
			uint32_t loads[NSTAGE] = { 0, 0, 0 };
			bool ok = !a.withhold;
			for (int64_t tA = blockIdx.x; tA < ntiles && ok; tA += 2 * G) {
				const int nslot = tA + G < ntiles ? 2 : 1;
				const uint16_t *E = a.sched.e[nslot - 1];
				for (int i = 0; i < a.sched.n[nslot - 1]; i++) {
					const uint16_t e = E[i];
					if (!se_load(e))
						continue;
					const int s = se_stage(e);
					// the stage's previous content has been released by its last use
					if (!mbar_wait(bar(B_EMPTY + s), (loads[s] & 1) ^ 1, s_abort, a.err, 1)) {
						ok = false;
						break;
					}
					mbar_expect_tx(bar(B_FULL + s), WBLOCK_BYTES);
					bulk_g2s(sbase + SM_W + s * WBLOCK_BYTES,
					         (const uint8_t *)a.wimg + (size_t)se_block(e) * WBLOCK_BYTES, WBLOCK_BYTES,
					         bar(B_FULL + s));
					loads[s]++;
				}
			}
			// copies in flight must land before the CTA leaves
			for (int s = 0; s < NSTAGE; s++)
				if (loads[s] > 0)
					mbar_drain(bar(B_FULL + s), (loads[s] - 1) & 1);
		}
	} else if (warp == 1) {
		// ---------------- MMA issuer: the pair's schedule, slot by slot within each layer
		if (lane == 0) {
			uint32_t loads[NSTAGE] = { 0, 0, 0 }, act_ph[2] = { 0, 0 };
			bool ok = true;
			for (int64_t tA = blockIdx.x; tA < ntiles && ok; tA += 2 * G) {
				const int nslot = tA + G < ntiles ? 2 : 1;
				const uint16_t *E = a.sched.e[nslot - 1];
				int i = 0;
				for (int layer = 0; layer < 4 && ok; layer++)
					for (int sl = 0; sl < nslot && ok; sl++) {
						// the slot's activations of this layer are in shared memory
						if (!mbar_wait(bar(B_ACT + sl), act_ph[sl], s_abort, a.err, 3)) {
							ok = false;
							break;
						}
						act_ph[sl] ^= 1;
						tc_fence_after();
						const uint32_t acc = tmem + (uint32_t)(sl * 256);
						const uint32_t act = sbase + SM_ACT + sl * ACT_BYTES;
						const int nkb = layer == 0 ? 1 : 4;
						for (int u = 0; u < nkb; u++, i++) {
							const uint16_t e = E[i];
							const int s = se_stage(e), j = se_kb(e);
							if (se_load(e)) {
								if (!mbar_wait(bar(B_FULL + s), loads[s] & 1, s_abort, a.err, 2)) {
									ok = false;
									break;
								}
								loads[s]++;
							}
							tc_fence_after();
							const uint32_t abase = act + j * ACT_KB_BYTES;
							const uint32_t bbase = sbase + SM_W + s * WBLOCK_BYTES;
							const int nk = layer == 0 ? 1 : KB / 16;
							for (int k = 0; k < nk; k++)
								mma_bf16_ss(acc, sdesc(abase + 32 * k), sdesc(bbase + 32 * k), (u | k) != 0);
							if (se_last(e))
								mma_commit(bar(B_EMPTY + s));
						}
						if (ok)
							mma_commit(bar(B_DONE + sl));
					}
			}
			// every MMA issued so far completes before the tensor memory is freed
			mma_commit(bar(B_FINAL));
			mbar_drain(bar(B_FINAL), 0);
		}
	} else {
		// ---------------- epilogue: 16 warps, warp (q = lane quarter, g = column group)
		const int e = warp - 2;
		const int q = warp & 3;
		const int g = __shfl_sync(0xffffffffu, e >> 2, 0);   // warp-uniform: constant-bank operands
		const int r = q * 32 + lane;                  // tile row of this thread
		const uint32_t lane_off = (uint32_t)(q * 32) << 16;
		uint32_t done_ph[2] = { 0, 0 }, head_ph[2] = { 0, 0 };
		const float b5 = a.ht[HT_B5];
		bool ok = true;
		for (int64_t tA = blockIdx.x; tA < ntiles && ok; tA += 2 * G) {
			const int nslot = tA + G < ntiles ? 2 : 1;
			// features of both tiles into act K-block 0 (chunks 0 and 1 of each row)
			for (int sl = 0; sl < nslot; sl++) {
				const int64_t row = (tA + sl * G) * TILE_M + r;
				if (g == 0) {
					uint4 c0 = make_uint4(0, 0, 0, 0), c1 = c0;
					if (row < a.n) {
						__align__(16) bf16 f[16];
						feature_row(a.states + 7 * row, f);
						c0 = *reinterpret_cast<uint4 *>(f);
						c1 = *reinterpret_cast<uint4 *>(f + 8);
					}
					uint8_t *act = sm + SM_ACT + sl * ACT_BYTES;
					*reinterpret_cast<uint4 *>(act + swz(r, 0)) = c0;
					*reinterpret_cast<uint4 *>(act + swz(r, 1)) = c1;
				}
				fence_async_smem();
				__syncwarp();
				if (lane == 0)
					mbar_arrive(bar(B_ACT + sl));
			}
			for (int layer = 0; layer < 4 && ok; layer++) {
				const float *bias = a.ht + layer * H;   // b_l / 2
				if (layer == 2 && g == 0) {
					// the next pair's state rows into L2 while this pair finishes, so that its
					// features do not wait on HBM at the pair boundary
					for (int sl = 0; sl < 2; sl++) {
						const int64_t row = (tA + 2 * G + sl * G) * TILE_M + r;
						if (row < a.n)
							asm volatile("prefetch.global.L2 [%0];" ::"l"(a.states + 7 * row));
					}
				}
				for (int sl = 0; sl < nslot; sl++) {
					// the biases of K-block 0 load while the accumulator is still being computed
					float bv[2][16];
#pragma unroll
					for (int i = 0; i < 4; i++)
						*reinterpret_cast<float4 *>(bv[0] + 4 * i) =
						    *(reinterpret_cast<const float4 *>(bias + g * 16) + i);
					if (!mbar_wait(bar(B_DONE + sl), done_ph[sl], s_abort, a.err, 4)) {
						ok = false;
						break;
					}
					done_ph[sl] ^= 1;
					tc_fence_after();
					uint8_t *act = sm + SM_ACT + sl * ACT_BYTES;
					float head = 0.f;
					// this warp's 16 columns j*64 + g*16 .. +15 of each K-block j; the tensor-memory
					// load and the biases of block j + 1 are in flight while block j is computed
					uint32_t rv[2][16];
					tmem_ld16_nw(tmem + lane_off + (uint32_t)(sl * 256 + g * 16), rv[0]);
					tmem_wait_ld();
#pragma unroll
					for (int j = 0; j < 4; j++) {
						if (j < 3) {
							tmem_ld16_nw(tmem + lane_off + (uint32_t)(sl * 256 + (j + 1) * KB + g * 16),
							             rv[(j + 1) & 1]);
#pragma unroll
							for (int i = 0; i < 4; i++)
								*reinterpret_cast<float4 *>(bv[(j + 1) & 1] + 4 * i) = *(
								    reinterpret_cast<const float4 *>(bias + (j + 1) * KB + g * 16) + i);
						}
						const int col = j * KB + g * 16;
						const float *bvj = bv[j & 1];
						const uint32_t *cur = rv[j & 1];
						uint32_t pk[8];
#pragma unroll
						for (int i = 0; i < 16; i += 2)
							pk[i / 2] = silu_pair(cur[i], cur[i + 1], bvj[i], bvj[i + 1]);
						if (layer < 3) {
							uint8_t *kb = act + j * ACT_KB_BYTES;
							*reinterpret_cast<uint4 *>(kb + swz(r, 2 * g)) = make_uint4(pk[0], pk[1], pk[2], pk[3]);
							*reinterpret_cast<uint4 *>(kb + swz(r, 2 * g + 1)) = make_uint4(pk[4], pk[5], pk[6], pk[7]);
						} else {
							float wv[16];
#pragma unroll
							for (int i = 0; i < 4; i++)
								*reinterpret_cast<float4 *>(wv + 4 * i) =
								    *(reinterpret_cast<const float4 *>(a.ht + HT_W5 + col) + i);
#pragma unroll
							for (int i = 0; i < 8; i++) {
								const __nv_bfloat162 hh = *reinterpret_cast<__nv_bfloat162 *>(&pk[i]);
								head = fmaf(__low2float(hh), wv[2 * i], head);
								head = fmaf(__high2float(hh), wv[2 * i + 1], head);
							}
						}
						if (j < 3)
							tmem_wait_ld();
					}
					tc_fence_before();
					if (layer < 3) {
						// the whole accumulator is read and the next layer's input written
						fence_async_smem();
						__syncwarp();
						if (lane == 0)
							mbar_arrive(bar(B_ACT + sl));
						continue;
					}
					// head: the accumulator is read and the act buffer is free (all MMAs of the
					// slot are complete), so its first 2 KB hold the column-group partial sums
					float *part = (float *)act;
					part[g * TILE_M + r] = head;
					__syncwarp();
					if (lane == 0)
						mbar_arrive(bar(B_HEAD + sl));
					if (g == 0) {
						if (!mbar_wait(bar(B_HEAD + sl), head_ph[sl], s_abort, a.err, 5)) {
							ok = false;
							break;
						}
						const float s = part[r] + part[TILE_M + r] + part[2 * TILE_M + r] + part[3 * TILE_M + r] + b5;
						const int64_t row = (tA + sl * G) * TILE_M + r;
						if (row < a.n)
							a.prob[row] = a.logits ? s : 1.f / (1.f + __expf(-s));
					}
					head_ph[sl] ^= 1;
				}
			}
		}
	}
	tc_fence_before();
	__syncthreads();
	if (warp == 0) {
		__syncwarp();
		tc_fence_after();
		asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, 512;" ::"r"(tmem) : "memory");
	}
}

__global__ void k_head_table(const float *params, int64_t off_b1, int64_t off_b2, int64_t off_b3, int64_t off_b4,
                             int64_t off_w5, int64_t off_b5, float *ht)
{
	const int i = blockIdx.x * blockDim.x + threadIdx.x;
	if (i >= HT_FLOATS)
		return;
	float v = 0.f;
	if (i < HT_W5) {
		const int l = i / H, c = i % H;
		const int64_t off = l == 0 ? off_b1 : (l == 1 ? off_b2 : (l == 2 ? off_b3 : off_b4));
		v = 0.5f * params[off + c];
	} else if (i < HT_B5) {
		v = params[off_w5 + (i - HT_W5)];
	} else if (i == HT_B5) {
		v = params[off_b5];
	}
	ht[i] = v;
}

// Weight images for the kernel above: block 0 = W1 (256 x 16, zero-padded to
// k = 64), blocks 1 + 4 (l - 1) + j = K-block j of W_{l+1}.  Each block is
// 256 rows x 128 bytes in the 128-byte swizzle layout.  Values are BF16(w) / 2
// (= BF16(w / 2) exactly), so the accumulator holds z / 2.
__global__ void k_weight_image(const float *params, int64_t off_w1, int64_t off_w2, int64_t off_w3, int64_t off_w4,
                               bf16 *img)
{
	const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;   // one 16-byte chunk
	const int64_t nchunk = (int64_t)NWBLOCK * H * 8;
	if (i >= nchunk)
		return;
	const int b = (int)(i / (H * 8));
	const int n = (int)((i / 8) % H);
	const int c = (int)(i % 8);
	__align__(16) bf16 v[8];
	for (int e = 0; e < 8; e++) {
		float w = 0.f;
		if (b == 0) {
			const int k = c * 8 + e;
			if (k < KIN)
				w = params[off_w1 + (int64_t)n * KIN + k];
		} else {
			const int l = (b - 1) / 4, j = (b - 1) % 4;
			const int64_t off = l == 0 ? off_w2 : (l == 1 ? off_w3 : off_w4);
			w = params[off + (int64_t)n * H + j * KB + c * 8 + e];
		}
		v[e] = __float2bfloat16_rn(0.5f * w);
	}
	uint8_t *dst = (uint8_t *)img + (size_t)b * WBLOCK_BYTES + swz(n, c);
	*reinterpret_cast<uint4 *>(dst) = *reinterpret_cast<uint4 *>(v);
}

} // namespace tc
