// pw_mlp_tc.cuh -- fused forward pass of the proposal network on the 5th-generation
// tensor cores (tcgen05 + tensor memory), sm_103a.  Included by pw_mlp.cu inside
// its anonymous namespace (uses H, KIN, bf16, silu, feature_row).
//
// One persistent CTA per SM walks 128-row tiles of states.  Per tile:
//   features -> act (smem, BF16)            epilogue warps
//   L1: act x W1^T -> acc0 (TMEM, FP32)     MMA thread, 1 instruction (K = 16)
//   E1: acc0 + b1, SiLU -> act              epilogue warps, 64 columns at a time
//   L2: act x W2^T -> acc1                  MMA thread, K-block j starts as soon as
//   E2 ...                                  E1 has written K-block j of act
//   L4 -> acc1; E4: SiLU, dot with w5, sigmoid -> prob
// Layers alternate between two 256-column accumulators so that the MMAs of
// layer l+1 run while the epilogue still reads layer l's accumulator.
// Weights stream through a 4-stage ring of 32 KB K-blocks (256 rows x 64 k),
// each a single bulk copy of an image that is already in the 128-byte-swizzle
// layout the MMA reads (built by k_weight_image).
//
// Roles (576 threads): warp 0 = weight producer and TMEM owner, warp 1 = MMA
// issuer, warps 2..17 = epilogue (warp w reads TMEM lanes 32 (w % 4) ..).
// Every wait is an mbarrier try_wait bounded by a wall-clock limit; on
// expiry the kernel records an error, stops all roles, waits (bounded) for
// its copies and MMAs in flight, frees its tensor memory and returns.

namespace tc {

constexpr int TILE_M = 128;
constexpr int KB = 64;                        // k per weight block / act K-block
constexpr int NSTAGE = 4;
constexpr int WBLOCK_BYTES = H * KB * 2;      // 32 KB: 256 rows x 128 bytes
constexpr int NWBLOCK = 1 + 3 * (H / KB);     // W1 (one block) + 4 blocks for each of W2..W4
constexpr int ACT_KB_BYTES = TILE_M * KB * 2; // 16 KB per act K-block
constexpr int NEPI_WARPS = 16;
constexpr int NTHREADS = (2 + NEPI_WARPS) * 32;
constexpr uint64_t WAIT_LIMIT_NS = 2000000000ull;   // 2 s per wait

// shared-memory map (offsets from a 1024-byte aligned base)
constexpr int SM_ACT = 0;                                        // 4 x 16 KB
constexpr int SM_W = SM_ACT + 4 * ACT_KB_BYTES;                  // NSTAGE x 32 KB
constexpr int SM_BIAS = SM_W + NSTAGE * WBLOCK_BYTES;            // 4 x 256 floats
constexpr int SM_W5 = SM_BIAS + 4 * H * 4;                       // 256 floats + b5
constexpr int SM_PART = SM_W5 + (H + 4) * 4;                     // 4 x 128 floats (head partial sums)
constexpr int SM_BAR = SM_PART + 4 * TILE_M * 4;                 // mbarriers
constexpr int NBAR = 2 * NSTAGE + 4 + 2 + 1 + 1;                 // full, empty, act, done, head, final
constexpr int SM_MISC = SM_BAR + NBAR * 8;                       // tmem base, abort flag
constexpr int SMEM_BYTES = SM_MISC + 16 + 1024;                  // + alignment slack

// barrier indices
constexpr int B_FULL = 0, B_EMPTY = NSTAGE, B_ACT = 2 * NSTAGE, B_DONE = B_ACT + 4, B_HEAD = B_DONE + 2,
              B_FINAL = B_HEAD + 1;

__device__ __forceinline__ uint32_t smem_u32(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(uint32_t bar, uint32_t count)
{
	asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_arrive(uint32_t bar)
{
	asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(bar) : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint32_t bar, uint32_t bytes)
{
	asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes) : "memory");
}
__device__ __forceinline__ bool mbar_test(uint32_t bar, uint32_t parity)
{
	uint32_t ok;
	asm volatile("{\n\t.reg .pred p;\n\t"
	             "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
	             "selp.u32 %0, 1, 0, p;\n\t}"
	             : "=r"(ok)
	             : "r"(bar), "r"(parity)
	             : "memory");
	return ok != 0;
}
__device__ __forceinline__ uint64_t now_ns()
{
	uint64_t t;
	asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
	return t;
}

// Waits for the phase of `parity` to complete.  Gives up when another role has
// aborted or after WAIT_LIMIT_NS, recording `where` in *err; returns false then.
__device__ __noinline__ bool mbar_wait(uint32_t bar, uint32_t parity, volatile int *abort_flag, int *err, int where)
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

__device__ __forceinline__ void bulk_g2s(uint32_t dst, const void *src, uint32_t bytes, uint32_t bar)
{
	asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(dst),
	             "l"(src), "r"(bytes), "r"(bar)
	             : "memory");
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

struct FwdArgs {
	const double *states;
	int64_t n;
	const bf16 *wimg;        // NWBLOCK images of WBLOCK_BYTES
	const float *params;     // FP32 parameter block
	int64_t off_b[4];
	int64_t off_w5, off_b5;
	float *prob;
	int *err;
};

__global__ void __launch_bounds__(NTHREADS, 1) k_mlp_forward_tc(FwdArgs a)
{
	extern __shared__ uint8_t smem_raw[];
	uint8_t *sm = (uint8_t *)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
	const uint32_t sbase = smem_u32(sm);
	float *s_bias = (float *)(sm + SM_BIAS);
	float *s_w5 = (float *)(sm + SM_W5);
	float *s_part = (float *)(sm + SM_PART);
	uint32_t *s_tmem = (uint32_t *)(sm + SM_MISC);
	volatile int *s_abort = (volatile int *)(sm + SM_MISC + 4);
	auto bar = [&](int i) { return sbase + SM_BAR + 8 * i; };

	const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
	const int64_t ntiles = (a.n + TILE_M - 1) / TILE_M;

	for (int i = threadIdx.x; i < 4 * H; i += NTHREADS)
		s_bias[i] = a.params[a.off_b[i / H] + (i % H)];
	for (int i = threadIdx.x; i < H + 1; i += NTHREADS)
		s_w5[i] = i < H ? a.params[a.off_w5 + i] : a.params[a.off_b5];
	if (threadIdx.x == 0) {
		for (int s = 0; s < NSTAGE; s++) {
			mbar_init(bar(B_FULL + s), 1);
			mbar_init(bar(B_EMPTY + s), 1);
		}
		for (int j = 0; j < 4; j++)
			mbar_init(bar(B_ACT + j), NEPI_WARPS);
		mbar_init(bar(B_DONE + 0), 1);
		mbar_init(bar(B_DONE + 1), 1);
		mbar_init(bar(B_HEAD), NEPI_WARPS);
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
		// ---------------- weight producer
		if (lane == 0) {
			uint32_t it = 0;
			int64_t last_it[NSTAGE];
			for (int s = 0; s < NSTAGE; s++)
				last_it[s] = -1;
			bool ok = true;
			for (int64_t t = blockIdx.x; t < ntiles && ok; t += gridDim.x) {
				for (int b = 0; b < NWBLOCK; b++, it++) {
					const int s = it % NSTAGE;
					if (!mbar_wait(bar(B_EMPTY + s), ((it / NSTAGE) & 1) ^ 1, s_abort, a.err, 1)) {
						ok = false;
						break;
					}
					mbar_expect_tx(bar(B_FULL + s), WBLOCK_BYTES);
					bulk_g2s(sbase + SM_W + s * WBLOCK_BYTES, (const uint8_t *)a.wimg + (size_t)b * WBLOCK_BYTES,
					         WBLOCK_BYTES, bar(B_FULL + s));
					last_it[s] = it;
				}
			}
			// copies in flight must land before the CTA leaves
			for (int s = 0; s < NSTAGE; s++)
				if (last_it[s] >= 0)
					mbar_drain(bar(B_FULL + s), (uint32_t)((last_it[s] / NSTAGE) & 1));
		}
	} else if (warp == 1) {
		// ---------------- MMA issuer
		if (lane == 0) {
			uint32_t it = 0, act_ph[4] = { 0, 0, 0, 0 };
			bool ok = true;
			for (int64_t t = blockIdx.x; t < ntiles && ok; t += gridDim.x) {
				for (int layer = 0; layer < 4 && ok; layer++) {
					const uint32_t acc = tmem + (uint32_t)((layer & 1) * 256);
					const int nkb = layer == 0 ? 1 : 4;
					for (int j = 0; j < nkb; j++, it++) {
						const int s = it % NSTAGE;
						if (!mbar_wait(bar(B_FULL + s), (it / NSTAGE) & 1, s_abort, a.err, 2) ||
						    !mbar_wait(bar(B_ACT + j), act_ph[j], s_abort, a.err, 3)) {
							ok = false;
							break;
						}
						act_ph[j] ^= 1;
						tc_fence_after();
						const uint32_t abase = sbase + SM_ACT + j * ACT_KB_BYTES;
						const uint32_t bbase = sbase + SM_W + s * WBLOCK_BYTES;
						const int nk = layer == 0 ? 1 : KB / 16;
						for (int k = 0; k < nk; k++)
							mma_bf16_ss(acc, sdesc(abase + 32 * k), sdesc(bbase + 32 * k), (j | k) != 0);
						mma_commit(bar(B_EMPTY + s));
					}
					if (ok)
						mma_commit(bar(B_DONE + (layer & 1)));
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
		const int g = e >> 2;
		const int r = q * 32 + lane;                  // tile row of this thread
		const uint32_t lane_off = (uint32_t)(q * 32) << 16;
		uint32_t done_ph[2] = { 0, 0 }, head_ph = 0;
		bool ok = true;
		for (int64_t t = blockIdx.x; t < ntiles && ok; t += gridDim.x) {
			const int64_t row = t * TILE_M + r;
			// features of this tile into act K-block 0 (chunks 0 and 1 of each row)
			if (g == 0) {
				uint4 c0 = make_uint4(0, 0, 0, 0), c1 = c0;
				if (row < a.n) {
					__align__(16) bf16 f[16];
					feature_row(a.states + 7 * row, f);
					c0 = *reinterpret_cast<uint4 *>(f);
					c1 = *reinterpret_cast<uint4 *>(f + 8);
				}
				*reinterpret_cast<uint4 *>(sm + SM_ACT + swz(r, 0)) = c0;
				*reinterpret_cast<uint4 *>(sm + SM_ACT + swz(r, 1)) = c1;
			}
			fence_async_smem();
			__syncwarp();
			if (lane == 0)
				mbar_arrive(bar(B_ACT + 0));
			float head = 0.f;
			for (int layer = 0; layer < 4; layer++) {
				const int ai = layer & 1;
				if (!mbar_wait(bar(B_DONE + ai), done_ph[ai], s_abort, a.err, 4)) {
					ok = false;
					break;
				}
				done_ph[ai] ^= 1;
				tc_fence_after();
				const float *bias = s_bias + layer * H;
				for (int j = 0; j < 4; j++) {
					const int col = j * KB + g * 16;
					float v[16];
					tmem_ld16(tmem + lane_off + (uint32_t)(ai * 256 + col), v);
					uint32_t pk[8];
#pragma unroll
					for (int i = 0; i < 16; i += 2) {
						const float h0 = silu(v[i] + bias[col + i]);
						const float h1 = silu(v[i + 1] + bias[col + i + 1]);
						pk[i / 2] = pack_bf16x2(h0, h1);
					}
					if (layer < 3) {
						uint8_t *kb = sm + SM_ACT + j * ACT_KB_BYTES;
						*reinterpret_cast<uint4 *>(kb + swz(r, 2 * g)) = make_uint4(pk[0], pk[1], pk[2], pk[3]);
						*reinterpret_cast<uint4 *>(kb + swz(r, 2 * g + 1)) = make_uint4(pk[4], pk[5], pk[6], pk[7]);
						fence_async_smem();
						tc_fence_before();
						__syncwarp();
						if (lane == 0)
							mbar_arrive(bar(B_ACT + j));
					} else {
#pragma unroll
						for (int i = 0; i < 8; i++) {
							const __nv_bfloat162 h = *reinterpret_cast<__nv_bfloat162 *>(&pk[i]);
							head = fmaf(__low2float(h), s_w5[col + 2 * i], head);
							head = fmaf(__high2float(h), s_w5[col + 2 * i + 1], head);
						}
					}
				}
			}
			if (!ok)
				break;
			// head: sum the four column groups of each row, add b5, sigmoid
			tc_fence_before();
			s_part[g * TILE_M + r] = head;
			__syncwarp();
			if (lane == 0)
				mbar_arrive(bar(B_HEAD));
			if (g == 0) {
				if (!mbar_wait(bar(B_HEAD), head_ph, s_abort, a.err, 5)) {
					ok = false;
					break;
				}
				const float s = s_part[r] + s_part[TILE_M + r] + s_part[2 * TILE_M + r] + s_part[3 * TILE_M + r] +
				                s_w5[H];
				if (row < a.n)
					a.prob[row] = 1.f / (1.f + __expf(-s));
			}
			head_ph ^= 1;
		}
	}
	tc_fence_before();
	__syncthreads();
	if (warp == 0) {
		tc_fence_after();
		asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, 512;" ::"r"(tmem) : "memory");
	}
}

// Weight images for the kernel above: block 0 = W1 (256 x 16, zero-padded to
// k = 64), blocks 1 + 4 (l - 1) + j = K-block j of W_{l+1}.  Each block is
// 256 rows x 128 bytes in the 128-byte swizzle layout.
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
		v[e] = __float2bfloat16_rn(w);
	}
	uint8_t *dst = (uint8_t *)img + (size_t)b * WBLOCK_BYTES + swz(n, c);
	*reinterpret_cast<uint4 *>(dst) = *reinterpret_cast<uint4 *>(v);
}

} // namespace tc
