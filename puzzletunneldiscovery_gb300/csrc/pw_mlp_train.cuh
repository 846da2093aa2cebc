// pw_mlp_train.cuh -- tcgen05 GEMMs of the proposal network's training step.
// Included by pw_mlp.cu inside its anonymous namespace, after pw_mlp_tc.cuh
// (uses the tc:: mbarrier / descriptor / MMA helpers, bf16, silu, dsilu).
//
// C[M x N] = sum_k A[m][k] B[n][k]: A and B row-major with k contiguous, loaded
// by TMA (cp.async.bulk.tensor, 128-byte swizzle) into a ring of
// 64-wide K-blocks (2 stages for the K = 256 layers, so that two CTAs share an
// SM and one's epilogue overlaps the other's MMAs; 4 for the batch-long K of
// the weight gradients); one elected thread issues tcgen05.mma (M = 128, N = NT,
// K = 16, BF16 in, FP32 accumulate in tensor memory); four epilogue warps read
// the accumulator (tcgen05.ld) and apply one of:
//   E_FWD: z = acc + bias -> Z (FP32), h = SiLU(z) -> Y (BF16, [M][N]) and Yt ([N][M])
//   E_DX:  g = acc * SiLU'(Z) -> Y (BF16, [M][N]) and Yt ([N][M])
//   E_DW:  C[z] = acc (FP32 partial tile of K split z = blockIdx.z; k_reduce_splits sums)
// The transposed copies let every GEMM of the step read K-major operands:
// forward H_l W_l^T, input gradient G W_l (B = W_l^T), weight gradient
// G^T X_l (A = G^T, B = X_l^T, K = batch).
//
// Roles (192 threads): warp 0 = TMA producer, warp 1 = MMA issuer and TMEM
// owner, warps 2..5 = epilogue.  Every wait is bounded (tc::mbar_wait).

namespace tt {

using namespace tc;

constexpr int BM = 128, BK = 64;
constexpr int NTHREADS = 192;
enum { E_FWD = 0, E_DX = 1, E_DW = 2 };

template <int NT, int STAGES>
struct Cfg {
	static constexpr int A_BYTES = BM * BK * 2;               // 16 KB
	static constexpr int B_BYTES = NT * BK * 2;               // NT rows x 128 bytes
	static constexpr int STAGE_BYTES = A_BYTES + B_BYTES;     // multiple of 1024
	static constexpr int SM_BAR = STAGES * STAGE_BYTES;
	static constexpr int NBAR = 2 * STAGES + 1;               // full, empty, done
	static constexpr int SM_MISC = SM_BAR + NBAR * 8;
	static constexpr int SMEM = SM_MISC + 16 + 1024;
	static constexpr int TMEM_COLS = NT < 32 ? 32 : NT;       // power of two >= 32
	static constexpr uint32_t IDESC = (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(NT >> 3) << 17) |
	                                  ((uint32_t)(BM >> 4) << 24);
	static_assert(NT % 16 == 0 && NT >= 16 && NT <= 256, "N tile of kind::f16 with M = 128");
	static_assert((A_BYTES % 1024) == 0 && (B_BYTES % 1024) == 0, "1024-byte aligned operand tiles");
	static_assert(NT == 16 || NT == 32 || NT == 64 || NT == 128 || NT == 256, "tensor memory allocation");
};

struct Args {
	int M, N, K;
	int k_split;           // K range of one blockIdx.z (multiple of BK)
	const float *bias;     // E_FWD
	float *Z;              // E_FWD: out; E_DX: in ([M][N] FP32)
	bf16 *Y;               // [M][N] BF16 out (E_FWD, E_DX)
	bf16 *Yt;              // [N][ldt] BF16 out (E_FWD, E_DX), may be null
	int64_t ldt;
	float *C;              // E_DW: [splits][M][N] FP32 partials
	int *err;
};

__device__ __forceinline__ void tma_load_2d(uint32_t dst, const CUtensorMap *map, int x, int y, uint32_t bar)
{
	asm volatile("cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], "
	             "[%4];" ::"r"(dst),
	             "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(bar)
	             : "memory");
}

__device__ __forceinline__ void mma_n(uint32_t d_tmem, uint64_t a, uint64_t b, uint32_t idesc, uint32_t accumulate)
{
	asm volatile("{\n\t.reg .pred p;\n\t"
	             "setp.ne.b32 p, %4, 0;\n\t"
	             "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(d_tmem),
	             "l"(a), "l"(b), "r"(idesc), "r"(accumulate)
	             : "memory");
}

template <int NT, int EPI, int STAGES>
__global__ void __launch_bounds__(NTHREADS, 1) k_gemm_tc(const __grid_constant__ CUtensorMap ta,
                                                         const __grid_constant__ CUtensorMap tb, Args p)
{
	typedef Cfg<NT, STAGES> C;
	extern __shared__ uint8_t smem_raw[];
	uint8_t *sm = (uint8_t *)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
	const uint32_t sbase = smem_u32(sm);
	uint32_t *s_tmem = (uint32_t *)(sm + C::SM_MISC);
	volatile int *s_abort = (volatile int *)(sm + C::SM_MISC + 4);
	auto bar = [&](int i) { return sbase + C::SM_BAR + 8 * i; };
	const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
	const int m0 = blockIdx.x * BM, n0 = blockIdx.y * NT;
	const int kbeg = blockIdx.z * p.k_split;
	const int kend = min(p.K, kbeg + p.k_split);
	const int nkb = kend > kbeg ? (kend - kbeg + BK - 1) / BK : 0;

	if (threadIdx.x == 0) {
		for (int s = 0; s < STAGES; s++) {
			mbar_init(bar(s), 1);
			mbar_init(bar(STAGES + s), 1);
		}
		mbar_init(bar(2 * STAGES), 1);
		*s_abort = 0;
		asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
	}
	if (warp == 1) {
		asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(s_tmem)),
		             "r"(C::TMEM_COLS)
		             : "memory");
		asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
	}
	tc_fence_before();
	__syncthreads();
	tc_fence_after();
	const uint32_t tmem = *s_tmem;

	if (warp == 0) {
		if (lane == 0) {
			int last = -1;
			for (int kb = 0; kb < nkb; kb++) {
				const int s = kb % STAGES;
				if (!mbar_wait(bar(STAGES + s), ((kb / STAGES) & 1) ^ 1, s_abort, p.err, 11))
					break;
				const uint32_t a_dst = sbase + s * C::STAGE_BYTES;
				mbar_expect_tx(bar(s), C::STAGE_BYTES);
				tma_load_2d(a_dst, &ta, kbeg + kb * BK, m0, bar(s));
				tma_load_2d(a_dst + C::A_BYTES, &tb, kbeg + kb * BK, n0, bar(s));
				last = kb;
			}
			// loads in flight land before the CTA leaves
			for (int kb = last - STAGES + 1 < 0 ? 0 : last - STAGES + 1; kb <= last; kb++)
				mbar_drain(bar(kb % STAGES), (uint32_t)((kb / STAGES) & 1));
		}
	} else if (warp == 1) {
		if (lane == 0) {
			bool ok = true;
			for (int kb = 0; kb < nkb; kb++) {
				const int s = kb % STAGES;
				if (!mbar_wait(bar(s), (kb / STAGES) & 1, s_abort, p.err, 12)) {
					ok = false;
					break;
				}
				tc_fence_after();
				const uint32_t a = sbase + s * C::STAGE_BYTES, b = a + C::A_BYTES;
				// the last block may be partial: its zero-filled tail adds nothing
				for (int k = 0; k < BK / 16; k++)
					mma_n(tmem, sdesc(a + 32 * k), sdesc(b + 32 * k), C::IDESC, (kb | k) != 0);
				mma_commit(bar(STAGES + s));
			}
			mma_commit(bar(2 * STAGES));
			if (!ok)
				mbar_drain(bar(2 * STAGES), 0);
		}
	} else {
		// epilogue: warp w reads TMEM lanes 32 (w % 4) .. and owns those tile rows
		const int q = warp & 3;
		const int r = q * 32 + lane;
		const int m = m0 + r;
		const uint32_t lane_off = (uint32_t)(q * 32) << 16;
		if (mbar_wait(bar(2 * STAGES), 0, s_abort, p.err, 13)) {
			tc_fence_after();
			const bool row_ok = m < p.M;
			for (int c0 = 0; c0 < NT; c0 += 16) {
				// every lane takes part in the warp-collective tensor-memory load
				__syncwarp();
				float v[16];
				if (nkb > 0)
					tmem_ld16(tmem + lane_off + (uint32_t)c0, v);
				else
					for (int i = 0; i < 16; i++)
						v[i] = 0.f;
				const int n = n0 + c0;
				if (!row_ok || n >= p.N)
					continue;
				if (EPI == E_DW) {
					// this K split's partial tile: C[blockIdx.z][m][n], summed by k_reduce_splits
					float4 *crow = reinterpret_cast<float4 *>(p.C + ((size_t)blockIdx.z * p.M + m) * p.N + n);
#pragma unroll
					for (int i = 0; i < 4; i++)
						crow[i] = make_float4(v[4 * i], v[4 * i + 1], v[4 * i + 2], v[4 * i + 3]);
					continue;
				}
				float o[16];
				float4 *z4 = reinterpret_cast<float4 *>(p.Z + (size_t)m * p.N + n);
				if (EPI == E_FWD) {
					float zb[16];
#pragma unroll
					for (int i = 0; i < 16; i++)
						zb[i] = v[i] + __ldg(p.bias + n + i);
#pragma unroll
					for (int i = 0; i < 4; i++)
						z4[i] = make_float4(zb[4 * i], zb[4 * i + 1], zb[4 * i + 2], zb[4 * i + 3]);
#pragma unroll
					for (int i = 0; i < 16; i++)
						o[i] = silu(zb[i]);
				} else {
#pragma unroll
					for (int i = 0; i < 4; i++) {
						const float4 z = z4[i];
						o[4 * i] = v[4 * i] * dsilu(z.x);
						o[4 * i + 1] = v[4 * i + 1] * dsilu(z.y);
						o[4 * i + 2] = v[4 * i + 2] * dsilu(z.z);
						o[4 * i + 3] = v[4 * i + 3] * dsilu(z.w);
					}
				}
				__align__(16) bf16 hb[16];
#pragma unroll
				for (int i = 0; i < 16; i++)
					hb[i] = __float2bfloat16_rn(o[i]);
				uint4 *yrow = reinterpret_cast<uint4 *>(p.Y + (size_t)m * p.N + n);
				yrow[0] = *reinterpret_cast<uint4 *>(hb);
				yrow[1] = *reinterpret_cast<uint4 *>(hb + 8);
				if (p.Yt)
#pragma unroll
					for (int i = 0; i < 16; i++)
						p.Yt[(size_t)(n + i) * p.ldt + m] = hb[i];
			}
		}
	}
	tc_fence_before();
	__syncthreads();
	if (warp == 1) {
		__syncwarp();
		tc_fence_after();
		asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(C::TMEM_COLS) : "memory");
	}
}

// out[i] = sum over the K splits of ws[s][i] (weight gradients).
__global__ void k_reduce_splits(const float *ws, int splits, int64_t n, float *out)
{
	const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
	if (i >= n)
		return;
	float acc = 0.f;
	for (int s = 0; s < splits; s++)
		acc += ws[(size_t)s * n + i];
	out[i] = acc;
}

// Output head backward over 64-row tiles, one thread per hidden unit k:
//   dw5[k] += sum_r g[r] H4[r][k],  db5 += sum_r g[r],
//   G4[r][k] = BF16(g[r] w5[k] SiLU'(Z4[r][k])) row-major and transposed.
// The transposed copy goes through a shared-memory tile so both stores coalesce.
__global__ void __launch_bounds__(256) k_head_backward_t(const bf16 *H4, const float *Z4, const float *g,
                                                         const float *w5, int64_t n, float *dw5, float *db5, bf16 *G4,
                                                         bf16 *G4t, int64_t ldt)
{
	constexpr int R = 64;
	__shared__ bf16 tile[R][H + 8];
	const int k = threadIdx.x;
	const float wk = w5[k];
	float acc = 0.f, dbs = 0.f;
	for (int64_t r0 = (int64_t)blockIdx.x * R; r0 < n; r0 += (int64_t)gridDim.x * R) {
		const int rows = (int)min((int64_t)R, n - r0);
		// 8 rows at a time so that their loads are in flight together
		for (int i0 = 0; i0 < rows; i0 += 8) {
			float gv[8], hv[8], zv[8];
#pragma unroll
			for (int j = 0; j < 8; j++) {
				const bool ok = i0 + j < rows;
				const size_t o = (size_t)(r0 + i0 + j) * H + k;
				gv[j] = ok ? g[r0 + i0 + j] : 0.f;
				hv[j] = ok ? __bfloat162float(H4[o]) : 0.f;
				zv[j] = ok ? Z4[o] : 0.f;
			}
#pragma unroll
			for (int j = 0; j < 8; j++) {
				if (i0 + j >= rows)
					break;
				acc = fmaf(gv[j], hv[j], acc);
				dbs += gv[j];
				const bf16 gk = __float2bfloat16_rn(gv[j] * wk * dsilu(zv[j]));
				G4[(size_t)(r0 + i0 + j) * H + k] = gk;
				tile[i0 + j][k] = gk;
			}
		}
		__syncthreads();
		// transposed: warp w writes columns w, w + 8, ...; lanes run along the rows
		const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
		for (int c = warp; c < H; c += 8)
			for (int i = lane; i < rows; i += 32)
				G4t[(size_t)c * ldt + r0 + i] = tile[i][c];
		__syncthreads();
	}
	atomicAdd(&dw5[k], acc);
	if (k == 0)
		atomicAdd(db5, dbs);
}

// Column sums of a BF16 [n x 256] matrix (bias gradients): lane l sums columns
// 8l .. 8l + 7 with 16-byte loads, 8 warps over interleaved rows, then a
// shared-memory reduction and one atomic per column and block.
__global__ void __launch_bounds__(256) k_colsum_v(const bf16 *G, int64_t n, int64_t rows_per_block, float *out)
{
	__shared__ float part[8][H];
	const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
	float acc[8] = { 0, 0, 0, 0, 0, 0, 0, 0 };
	const int64_t r0 = blockIdx.x * rows_per_block, r1 = min(n, r0 + rows_per_block);
	for (int64_t r = r0 + warp; r < r1; r += 8) {
		const uint4 v = *reinterpret_cast<const uint4 *>(G + (size_t)r * H + 8 * lane);
		const bf16 *b = reinterpret_cast<const bf16 *>(&v);
#pragma unroll
		for (int i = 0; i < 8; i++)
			acc[i] += __bfloat162float(b[i]);
	}
#pragma unroll
	for (int i = 0; i < 8; i++)
		part[warp][8 * lane + i] = acc[i];
	__syncthreads();
	float s = 0.f;
	for (int w = 0; w < 8; w++)
		s += part[w][threadIdx.x];
	atomicAdd(&out[threadIdx.x], s);
}

} // namespace tt
