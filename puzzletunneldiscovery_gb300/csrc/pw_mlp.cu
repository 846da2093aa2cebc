// pw_mlp.cu -- the learned proposal: a BF16 MLP trained on exact collision labels.
//
// The reference has no such network for this path (its learned part predicts
// surface heat maps, src/hg); this is the engine's own surrogate.
//   features (9 of 16): translation, first two columns of R(q)      [BF16]
//   4 hidden layers of width 256, SiLU                               [BF16 weights and activations]
//   output: sigmoid(w5 . h4 + b5) = P(state is collision free)       [FP32 accumulation everywhere]
// Training: binary cross-entropy, Adam; master weights and moments FP32.
// GEMMs are hand-written tensor-core kernels (mma.sync BF16 m16n8k16 with FP32
// accumulation) with fused bias + SiLU epilogues.
#include <cuda.h>
#include <cudaTypedefs.h>
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cmath>
#include <cstring>
#include <random>
#include <string>
#include <vector>

#include "pw_async.cuh"
#include "pw_internal.cuh"
#include "pw_mlp.h"

namespace {

constexpr int H = 256;        // hidden width
constexpr int KIN = 16;       // padded input width (9 features)
constexpr int NLAYER = 4;     // hidden layers

typedef __nv_bfloat16 bf16;

// ------------------------------------------------------------------ GEMM
//
// C[M x N] = sum_k A(m, k) B(n, k), A and B in BF16, FP32 accumulation.
// A_KCONT: A stored [M][K] (k contiguous), else [K][M].  Same for B ([N][K] or [K][N]).
// Tiles 128 x 128 x 32, 8 warps (2 x 4), double-buffered cp.async, ldmatrix.
constexpr int BM = 128, BN = 128, BK = 32;
constexpr int PAD = 8;        // halves of padding per smem row

enum Epi {
	EPI_BIAS_SILU = 0,   // Z = acc + bias[n] -> Zout (FP32), Y = SiLU(Z) -> bf16
	EPI_DSILU = 1,       // G = acc * SiLU'(Z[m, n]) -> bf16
	EPI_ATOMIC_F32 = 2,  // Cf[m, n] += acc (split-K partial sums)
};

struct GemmArgs {
	const bf16 *A, *B;
	int M, N, K;
	int lda, ldb;          // leading dimensions (elements)
	int k_split;           // K range per blockIdx.z
	const float *bias;     // EPI_BIAS_SILU
	float *Zout;           // EPI_BIAS_SILU: pre-activations (may be null)
	const float *Zin;      // EPI_DSILU
	bf16 *Y;               // bf16 output (ldc = N)
	float *Cf;             // EPI_ATOMIC_F32 output (ldc = N)
};

__device__ __forceinline__ void cp_async16(void *smem, const void *gmem, bool pred)
{
	const unsigned s = (unsigned)__cvta_generic_to_shared(smem);
	const int sz = pred ? 16 : 0;
	asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;\n" ::"r"(s), "l"(gmem), "r"(sz));
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::); }
template <int N>
__device__ __forceinline__ void cp_async_wait() { asm volatile("cp.async.wait_group %0;\n" ::"n"(N)); }

__device__ __forceinline__ void ldsm_x4(unsigned &r0, unsigned &r1, unsigned &r2, unsigned &r3, const void *p)
{
	const unsigned a = (unsigned)__cvta_generic_to_shared(p);
	asm volatile("ldmatrix.sync.aligned.m8n8.x4.shared.b16 {%0,%1,%2,%3}, [%4];\n"
	             : "=r"(r0), "=r"(r1), "=r"(r2), "=r"(r3) : "r"(a));
}
__device__ __forceinline__ void ldsm_x4_t(unsigned &r0, unsigned &r1, unsigned &r2, unsigned &r3, const void *p)
{
	const unsigned a = (unsigned)__cvta_generic_to_shared(p);
	asm volatile("ldmatrix.sync.aligned.m8n8.x4.trans.shared.b16 {%0,%1,%2,%3}, [%4];\n"
	             : "=r"(r0), "=r"(r1), "=r"(r2), "=r"(r3) : "r"(a));
}
__device__ __forceinline__ void ldsm_x2(unsigned &r0, unsigned &r1, const void *p)
{
	const unsigned a = (unsigned)__cvta_generic_to_shared(p);
	asm volatile("ldmatrix.sync.aligned.m8n8.x2.shared.b16 {%0,%1}, [%2];\n" : "=r"(r0), "=r"(r1) : "r"(a));
}
__device__ __forceinline__ void ldsm_x2_t(unsigned &r0, unsigned &r1, const void *p)
{
	const unsigned a = (unsigned)__cvta_generic_to_shared(p);
	asm volatile("ldmatrix.sync.aligned.m8n8.x2.trans.shared.b16 {%0,%1}, [%2];\n" : "=r"(r0), "=r"(r1) : "r"(a));
}
__device__ __forceinline__ void mma_bf16(float *d, unsigned a0, unsigned a1, unsigned a2, unsigned a3, unsigned b0,
                                         unsigned b1)
{
	asm volatile("mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
	             "{%0,%1,%2,%3};\n"
	             : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
	             : "r"(a0), "r"(a1), "r"(a2), "r"(a3), "r"(b0), "r"(b1));
}

// SiLU through one hardware tanh: silu(z) = z sigmoid(z) = h + h tanh(h), h = z / 2.
// tanh.approx.f32 has a relative error near 2^-11, below the BF16 rounding that follows.
__device__ __forceinline__ float tanh_fast(float x)
{
	float y;
	asm("tanh.approx.f32 %0, %1;" : "=f"(y) : "f"(x));
	return y;
}
__device__ __forceinline__ float silu(float z)
{
	const float h = 0.5f * z;
	return fmaf(h, tanh_fast(h), h);
}
// d silu / dz = s (1 + z (1 - s)), s = sigmoid(z) = (1 + tanh(z / 2)) / 2
__device__ __forceinline__ float dsilu(float z)
{
	const float s = fmaf(0.5f, tanh_fast(0.5f * z), 0.5f);
	return s * (1.f + z * (1.f - s));
}

// Shared-memory tile of a K-contiguous operand: [rows][BK + PAD]; of an
// M/N-contiguous operand: [BK][rows + PAD].
template <bool KCONT, int ROWS>
struct TileLayout {
	static constexpr int elems = KCONT ? ROWS * (BK + PAD) : BK * (ROWS + PAD);
};

// Copy one BK slice of a ROWS-row operand into shared memory (256 threads, 16-byte chunks).
template <bool KCONT, int ROWS>
__device__ __forceinline__ void load_tile(bf16 *s, const bf16 *g, int ld, int row0, int nrows, int k0, int kend)
{
	if (KCONT) {
		// ROWS x BK halves = ROWS * 4 chunks of 8 halves
		for (int c = threadIdx.x; c < ROWS * (BK / 8); c += 256) {
			const int r = c / (BK / 8), kk = (c % (BK / 8)) * 8;
			const bool ok = (row0 + r) < nrows && (k0 + kk) < kend;
			const bf16 *src = ok ? g + (size_t)(row0 + r) * ld + k0 + kk : g;
			cp_async16(s + r * (BK + PAD) + kk, src, ok);
		}
	} else {
		// BK x ROWS halves, rows contiguous
		for (int c = threadIdx.x; c < BK * (ROWS / 8); c += 256) {
			const int kk = c / (ROWS / 8), r = (c % (ROWS / 8)) * 8;
			const bool ok = (k0 + kk) < kend && (row0 + r) < nrows;
			const bf16 *src = ok ? g + (size_t)(k0 + kk) * ld + row0 + r : g;
			cp_async16(s + kk * (ROWS + PAD) + r, src, ok);
		}
	}
}

template <bool A_KCONT, bool B_KCONT, int EPI>
__global__ void __launch_bounds__(256) k_gemm(GemmArgs p)
{
	__shared__ __align__(16) bf16 sA[2][TileLayout<A_KCONT, BM>::elems];
	__shared__ __align__(16) bf16 sB[2][TileLayout<B_KCONT, BN>::elems];
	const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
	const int wm = warp >> 2, wn = warp & 3;     // 2 x 4 warps, each 64 x 32
	const int m0 = blockIdx.y * BM, n0 = blockIdx.x * BN;
	const int kbeg = blockIdx.z * p.k_split;
	const int kend = min(p.K, kbeg + p.k_split);
	float acc[4][4][4];
#pragma unroll
	for (int i = 0; i < 4; i++)
#pragma unroll
		for (int j = 0; j < 4; j++)
#pragma unroll
			for (int r = 0; r < 4; r++)
				acc[i][j][r] = 0.f;
	const int nk = (kend - kbeg + BK - 1) / BK;
	if (nk > 0) {
		load_tile<A_KCONT, BM>(sA[0], p.A, p.lda, m0, p.M, kbeg, kend);
		load_tile<B_KCONT, BN>(sB[0], p.B, p.ldb, n0, p.N, kbeg, kend);
	}
	cp_async_commit();
	for (int t = 0; t < nk; t++) {
		const int cur = t & 1;
		if (t + 1 < nk) {
			load_tile<A_KCONT, BM>(sA[cur ^ 1], p.A, p.lda, m0, p.M, kbeg + (t + 1) * BK, kend);
			load_tile<B_KCONT, BN>(sB[cur ^ 1], p.B, p.ldb, n0, p.N, kbeg + (t + 1) * BK, kend);
		}
		cp_async_commit();
		cp_async_wait<1>();
		__syncthreads();
		const bf16 *a = sA[cur], *b = sB[cur];
#pragma unroll
		for (int ks = 0; ks < BK; ks += 16) {
			unsigned af[4][4], bfr[4][2];
#pragma unroll
			for (int i = 0; i < 4; i++) {
				const int mr = wm * 64 + i * 16;
				if (A_KCONT) {
					const bf16 *ptr = a + (mr + (lane & 15)) * (BK + PAD) + ks + (lane >> 4) * 8;
					ldsm_x4(af[i][0], af[i][1], af[i][2], af[i][3], ptr);
				} else {
					// [k][m] storage: transpose on load
					const bf16 *ptr = a + (ks + (lane & 7) + ((lane >> 4) << 3)) * (BM + PAD) + mr + ((lane >> 3) & 1) * 8;
					ldsm_x4_t(af[i][0], af[i][1], af[i][2], af[i][3], ptr);
				}
			}
#pragma unroll
			for (int j = 0; j < 4; j++) {
				const int nr = wn * 32 + j * 8;
				if (B_KCONT) {
					const bf16 *ptr = b + (nr + (lane & 7)) * (BK + PAD) + ks + ((lane >> 3) & 1) * 8;
					ldsm_x2(bfr[j][0], bfr[j][1], ptr);
				} else {
					const bf16 *ptr = b + (ks + (lane & 15)) * (BN + PAD) + nr;
					ldsm_x2_t(bfr[j][0], bfr[j][1], ptr);
				}
			}
#pragma unroll
			for (int i = 0; i < 4; i++)
#pragma unroll
				for (int j = 0; j < 4; j++)
					mma_bf16(acc[i][j], af[i][0], af[i][1], af[i][2], af[i][3], bfr[j][0], bfr[j][1]);
		}
		__syncthreads();
	}
	// epilogue: acc[i][j] covers rows m0 + wm*64 + i*16 + {g, g+8}, cols n0 + wn*32 + j*8 + 2c + {0,1}
	const int g = lane >> 2, c4 = lane & 3;
#pragma unroll
	for (int i = 0; i < 4; i++)
#pragma unroll
		for (int j = 0; j < 4; j++)
#pragma unroll
			for (int h = 0; h < 2; h++) {
				const int m = m0 + wm * 64 + i * 16 + g + h * 8;
				const int n = n0 + wn * 32 + j * 8 + 2 * c4;
				if (m >= p.M || n >= p.N)
					continue;
				float v0 = acc[i][j][2 * h], v1 = acc[i][j][2 * h + 1];
				const size_t o = (size_t)m * p.N + n;
				if (EPI == EPI_BIAS_SILU) {
					v0 += p.bias[n];
					v1 += p.bias[n + 1];
					if (p.Zout) {
						p.Zout[o] = v0;
						p.Zout[o + 1] = v1;
					}
					*reinterpret_cast<__nv_bfloat162 *>(p.Y + o) = __floats2bfloat162_rn(silu(v0), silu(v1));
				} else if (EPI == EPI_DSILU) {
					v0 *= dsilu(p.Zin[o]);
					v1 *= dsilu(p.Zin[o + 1]);
					*reinterpret_cast<__nv_bfloat162 *>(p.Y + o) = __floats2bfloat162_rn(v0, v1);
				} else {
					atomicAdd(p.Cf + o, v0);
					atomicAdd(p.Cf + o + 1, v1);
				}
			}
}

// ------------------------------------------------------------------ small kernels

// Features of a state: translation and the first two columns of R(q), in FP32
// with every operation rounded separately (no contraction), then BF16.
__device__ __forceinline__ void feature_values(const double *q, float f[9])
{
	const float w = (float)q[3], x = (float)q[4], y = (float)q[5], z = (float)q[6];
	auto m = [](float a, float b) { return __fmul_rn(a, b); };
	auto a = [](float u, float v) { return __fadd_rn(u, v); };
	auto s = [](float u, float v) { return __fsub_rn(u, v); };
	f[0] = (float)q[0];
	f[1] = (float)q[1];
	f[2] = (float)q[2];
	f[3] = s(1.f, m(2.f, a(m(y, y), m(z, z))));
	f[4] = m(2.f, a(m(x, y), m(w, z)));
	f[5] = m(2.f, s(m(x, z), m(w, y)));
	f[6] = m(2.f, s(m(x, y), m(w, z)));
	f[7] = s(1.f, m(2.f, a(m(x, x), m(z, z))));
	f[8] = m(2.f, a(m(y, z), m(w, x)));
}

__device__ __forceinline__ void feature_row(const double *q, bf16 *o)
{
	float f[9];
	feature_values(q, f);
#pragma unroll
	for (int k = 0; k < KIN; k++)
		o[k] = __float2bfloat16_rn(k < 9 ? f[k] : 0.f);
}

__global__ void k_features(const double *states, int64_t n, bf16 *X)
{
	const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
	if (i >= n)
		return;
	feature_row(states + 7 * i, X + i * KIN);
}

// Output layer: s = w5 . h + b5, p = sigmoid(s).  One warp per row.
__global__ void k_head_forward(const bf16 *Hl, const float *w5, const float *b5, int64_t n, float *logit, float *prob)
{
	const int64_t row = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
	const int lane = threadIdx.x & 31;
	if (row >= n)
		return;
	const bf16 *h = Hl + row * H;
	float s = 0.f;
	for (int k = lane; k < H; k += 32)
		s += __bfloat162float(h[k]) * w5[k];
	for (int o = 16; o > 0; o >>= 1)
		s += __shfl_down_sync(0xffffffffu, s, o);
	if (lane == 0) {
		s += b5[0];
		if (logit)
			logit[row] = s;
		if (prob)
			prob[row] = 1.f / (1.f + __expf(-s));
	}
}

// Binary cross-entropy on logits; g = dL/ds = (sigmoid(s) - y) / n; loss summed.
__global__ void k_head_loss(const float *logit, const uint8_t *label, int64_t n, float *g, float *loss)
{
	const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
	float l = 0.f;
	if (i < n) {
		const float s = logit[i], y = label[i] ? 1.f : 0.f;
		const float p = 1.f / (1.f + __expf(-s));
		g[i] = (p - y) / (float)n;
		// log(1 + e^-|s|) + max(s, 0) - y s
		l = log1pf(__expf(-fabsf(s))) + fmaxf(s, 0.f) - y * s;
	}
	for (int o = 16; o > 0; o >>= 1)
		l += __shfl_down_sync(0xffffffffu, l, o);
	if ((threadIdx.x & 31) == 0)
		atomicAdd(loss, l / (float)n);
}

// dW5 += g . h4, db5 += sum g, and G4 = (g w5^T) * SiLU'(Z4) in BF16.
__global__ void k_head_backward(const bf16 *H4, const float *Z4, const float *g, const float *w5, int64_t n,
                                float *dw5, float *db5, bf16 *G4, bf16 *G4t = nullptr, int64_t ldt = 0)
{
	__shared__ float sw[H];
	for (int k = threadIdx.x; k < H; k += blockDim.x)
		sw[k] = 0.f;
	__syncthreads();
	const int lane = threadIdx.x & 31;
	float db = 0.f;
	for (int64_t row = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5; row < n;
	     row += ((int64_t)gridDim.x * blockDim.x) >> 5) {
		const float gi = g[row];
		db += lane == 0 ? gi : 0.f;
		for (int k = lane; k < H; k += 32) {
			const size_t o = (size_t)row * H + k;
			atomicAdd(&sw[k], gi * __bfloat162float(H4[o]));
			const bf16 gk = __float2bfloat16_rn(gi * w5[k] * dsilu(Z4[o]));
			G4[o] = gk;
			if (G4t)
				G4t[(size_t)k * ldt + row] = gk;
		}
	}
	__syncthreads();
	for (int k = threadIdx.x; k < H; k += blockDim.x)
		atomicAdd(&dw5[k], sw[k]);
	for (int o = 16; o > 0; o >>= 1)
		db += __shfl_down_sync(0xffffffffu, db, o);
	if (lane == 0)
		atomicAdd(db5, db);
}

// Column sums of a BF16 [n x H] matrix into FP32 (bias gradients).
__global__ void k_colsum(const bf16 *G, int64_t n, float *out)
{
	const int col = threadIdx.x;   // blockDim.x == H
	float s = 0.f;
	for (int64_t r = blockIdx.x; r < n; r += gridDim.x)
		s += __bfloat162float(G[(size_t)r * H + col]);
	atomicAdd(&out[col], s);
}

// Adam on FP32 masters; refreshes the BF16 copy (and its transpose when given).
__global__ void k_adam(float *w, const float *grad, float *m, float *v, int64_t n, float lr, float b1, float b2,
                       float eps, float c1, float c2, bf16 *wb, bf16 *wbt, int rows, int cols)
{
	const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
	if (i >= n)
		return;
	const float gr = grad[i];
	const float mi = b1 * m[i] + (1.f - b1) * gr;
	const float vi = b2 * v[i] + (1.f - b2) * gr * gr;
	m[i] = mi;
	v[i] = vi;
	const float wi = w[i] - lr * (mi / c1) / (sqrtf(vi / c2) + eps);
	w[i] = wi;
	if (wb)
		wb[i] = __float2bfloat16_rn(wi);
	if (wbt) {
		const int r = (int)(i / cols), c = (int)(i % cols);
		wbt[(size_t)c * rows + r] = __float2bfloat16_rn(wi);
	}
}

__global__ void k_to_bf16(const float *w, int64_t n, bf16 *wb, bf16 *wbt, int rows, int cols)
{
	const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
	if (i >= n)
		return;
	wb[i] = __float2bfloat16_rn(w[i]);
	if (wbt) {
		const int r = (int)(i / cols), c = (int)(i % cols);
		wbt[(size_t)c * rows + r] = __float2bfloat16_rn(w[i]);
	}
}

#include "pw_mlp_tc.cuh"
#include "pw_mlp_train.cuh"

// Zero-padded 64-wide input rows (the tcgen05 GEMM reads K-blocks of 64) and
// the transposed 16-wide features (the B operand of the first weight gradient).
__global__ void k_features64(const double *states, int64_t n, bf16 *X64, bf16 *Xt, int64_t ldt)
{
	const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
	if (i >= n)
		return;
	__align__(16) bf16 f[KIN];
	feature_row(states + 7 * i, f);
	uint4 *o = reinterpret_cast<uint4 *>(X64 + i * 64);
	o[0] = *reinterpret_cast<uint4 *>(f);
	o[1] = *reinterpret_cast<uint4 *>(f + 8);
	for (int c = 2; c < 8; c++)
		o[c] = make_uint4(0, 0, 0, 0);
	for (int k = 0; k < KIN; k++)
		Xt[(size_t)k * ldt + i] = f[k];
}

// W1 [256][16] -> BF16 [256][64], zero-padded.
__global__ void k_w1_pad(const float *W1, bf16 *out)
{
	const int i = blockIdx.x * blockDim.x + threadIdx.x;
	if (i >= H * 64)
		return;
	const int r = i / 64, c = i % 64;
	out[i] = __float2bfloat16_rn(c < KIN ? W1[r * KIN + c] : 0.f);
}

// ------------------------------------------------------------------ top-k selection
//
// Scores are floats mapped to 32-bit keys that order like the values (sign
// bit flipped for non-negative values, all bits flipped for negative ones).
// Three histogram passes over 11, 11 and 10 bits of the key (block-private
// shared-memory counters) find the key of the k-th largest score exactly; a
// compaction pass gathers the states at or above it.
__device__ __forceinline__ uint32_t score_key(float v)
{
	const uint32_t b = __float_as_uint(v);
	return (b & 0x80000000u) ? ~b : (b | 0x80000000u);
}
constexpr int SEL_BITS[3] = { 11, 11, 10 };
constexpr int SEL_SHIFT[3] = { 21, 10, 0 };

__global__ void k_score_hist(const float *score, int64_t n, int shift, int bits, uint32_t prefix, int prefix_shift,
                             unsigned long long *hist)
{
	__shared__ unsigned int sh[2048];
	const int nb = 1 << bits;
	for (int i = threadIdx.x; i < nb; i += blockDim.x)
		sh[i] = 0;
	__syncthreads();
	for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
		const uint32_t b = score_key(score[i]);
		if (prefix_shift >= 32 || (b >> prefix_shift) == prefix)
			atomicAdd(&sh[(b >> shift) & (nb - 1)], 1u);
	}
	__syncthreads();
	for (int i = threadIdx.x; i < nb; i += blockDim.x)
		if (sh[i])
			atomicAdd(&hist[i], (unsigned long long)sh[i]);
}

__global__ void k_select_states(const float *score, const double *states, int64_t n, uint32_t thr_bits,
                                double *out, int64_t capacity, unsigned long long *count)
{
	const int lane = threadIdx.x & 31;
	for (int64_t base = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) - lane; base < n;
	     base += (int64_t)gridDim.x * blockDim.x) {
		const int64_t i = base + lane;
		const bool take = i < n && score_key(score[i]) >= thr_bits;
		const unsigned mask = __ballot_sync(0xffffffffu, take);
		unsigned long long at = 0;
		if (lane == 0 && mask)
			at = atomicAdd(count, (unsigned long long)__popc(mask));
		at = __shfl_sync(0xffffffffu, at, 0);
		if (take) {
			const int64_t o = (int64_t)at + __popc(mask & ((1u << lane) - 1));
			if (o < capacity)
				for (int c = 0; c < 7; c++)
					out[7 * o + c] = states[7 * i + c];
		}
	}
}

} // namespace

// ------------------------------------------------------------------ the network object

struct pw_mlp {
	int device = 0;
	// parameter layout in one FP32 block: W1 [H x KIN], b1, W2..W4 [H x H], b2..b4, w5 [H], b5
	size_t off_w[NLAYER], off_b[NLAYER], off_w5 = 0, off_b5 = 0, nparam = 0;
	DeviceBuffer params, grads, m1, m2;
	DeviceBuffer wbf, wbft;      // BF16 weights and transposes (hidden layers)
	size_t off_wb[NLAYER];
	DeviceBuffer acts, zs, gbuf, gbuf2, head, misc;
	DeviceBuffer wimg;           // swizzled BF16 weight images of the tcgen05 forward kernel
	// tcgen05 training: padded inputs, transposed activations / gradients, split-K partials
	DeviceBuffer x64, xt, ht, gt, w1p, dw_ws;
	int64_t tcap = 0;            // rows (multiple of 128) of the training buffers above
	bool mma_training = false;   // train with the mma.sync kernels instead
	bool withhold_next = false;  // the next tcgen05 forward launch issues no weight copies
	bool wimg_dirty = true;
	std::vector<float> ht_host;  // the epilogue constants (tc::HT_*), passed in each forward launch's parameters
	int num_sms = 1;
	int64_t cap = 0;             // rows the activation buffers hold
	int64_t step = 0;
	float b1 = 0.9f, b2 = 0.999f, eps = 1e-8f;
};

static int in_dim(int l) { return l == 0 ? KIN : H; }

static int mlp_reserve(pw_mlp *m, int64_t rows)
{
	if (rows <= m->cap)
		return PW_OK;
	const int64_t r = ((rows + BM - 1) / BM) * BM;
	PW_CUDA(m->acts.reserve(sizeof(bf16) * (size_t)r * (KIN + NLAYER * H)));   // X0 and H1..H4
	PW_CUDA(m->zs.reserve(sizeof(float) * (size_t)r * NLAYER * H));           // Z1..Z4
	PW_CUDA(m->gbuf.reserve(sizeof(bf16) * (size_t)r * H));
	PW_CUDA(m->gbuf2.reserve(sizeof(bf16) * (size_t)r * H));
	PW_CUDA(m->head.reserve(sizeof(float) * (size_t)r * 2));                  // logits, dL/ds
	m->cap = r;
	return PW_OK;
}

static bf16 *act(pw_mlp *m, int l)   // 0: X0 [cap x KIN], l >= 1: H_l [cap x H]
{
	bf16 *base = (bf16 *)m->acts.ptr;
	return l == 0 ? base : base + (size_t)m->cap * KIN + (size_t)(l - 1) * m->cap * H;
}
static float *zbuf(pw_mlp *m, int l) { return (float *)m->zs.ptr + (size_t)(l - 1) * m->cap * H; }

extern "C" int pw_mlp_create(pw_mlp **out, int device, uint64_t seed)
{
	if (!out)
		return pw_fail(PW_ERR_INVALID_ARG, "pw_mlp_create: out is NULL");
	PW_CUDA(cudaSetDevice(device));
	pw_mlp *m = new pw_mlp();
	m->device = device;
	size_t o = 0, ob = 0;
	for (int l = 0; l < NLAYER; l++) {
		m->off_w[l] = o;
		o += (size_t)H * in_dim(l);
		m->off_b[l] = o;
		o += H;
		m->off_wb[l] = ob;
		ob += (size_t)H * in_dim(l);
	}
	m->off_w5 = o;
	o += H;
	m->off_b5 = o;
	o += 1;
	m->nparam = o;
	int rc = PW_OK;
	auto chk = [&](cudaError_t e) {
		if (e != cudaSuccess && rc == PW_OK)
			rc = pw_cuda_fail(e, "pw_mlp_create");
	};
	chk(m->params.reserve(sizeof(float) * o));
	chk(m->grads.reserve(sizeof(float) * o));
	chk(m->m1.reserve(sizeof(float) * o));
	chk(m->m2.reserve(sizeof(float) * o));
	chk(m->wbf.reserve(sizeof(bf16) * ob));
	chk(m->wbft.reserve(sizeof(bf16) * ob));
	chk(m->misc.reserve(64));
	chk(cudaMemset(m->misc.ptr, 0, 64));
	chk(cudaDeviceGetAttribute(&m->num_sms, cudaDevAttrMultiProcessorCount, device));
	if (rc) {
		delete m;
		return rc;
	}
	// He-uniform weights, zero biases (host RNG, seeded)
	std::vector<float> h(o, 0.f);
	std::mt19937_64 rng(seed);
	for (int l = 0; l < NLAYER; l++) {
		const float a = std::sqrt(6.f / (float)(l == 0 ? 9 : H));
		std::uniform_real_distribution<float> U(-a, a);
		for (int r = 0; r < H; r++)
			for (int c = 0; c < in_dim(l); c++)
				h[m->off_w[l] + (size_t)r * in_dim(l) + c] = (l == 0 && c >= 9) ? 0.f : U(rng);
	}
	{
		const float a = std::sqrt(6.f / (float)H);
		std::uniform_real_distribution<float> U(-a, a);
		for (int k = 0; k < H; k++)
			h[m->off_w5 + k] = 0.1f * U(rng);
	}
	chk(cudaMemcpy(m->params.ptr, h.data(), sizeof(float) * o, cudaMemcpyHostToDevice));
	chk(cudaMemset(m->m1.ptr, 0, sizeof(float) * o));
	chk(cudaMemset(m->m2.ptr, 0, sizeof(float) * o));
	for (int l = 0; l < NLAYER; l++) {
		const int64_t nw = (int64_t)H * in_dim(l);
		k_to_bf16<<<(unsigned)((nw + 255) / 256), 256>>>((float *)m->params.ptr + m->off_w[l], nw,
		                                                 (bf16 *)m->wbf.ptr + m->off_wb[l],
		                                                 (bf16 *)m->wbft.ptr + m->off_wb[l], H, in_dim(l));
	}
	chk(cudaGetLastError());
	chk(cudaDeviceSynchronize());
	if (rc) {
		delete m;
		return rc;
	}
	*out = m;
	return PW_OK;
}

extern "C" int pw_mlp_destroy(pw_mlp *m)
{
	if (m) {
		cudaSetDevice(m->device);
		delete m;
	}
	return PW_OK;
}

extern "C" int64_t pw_mlp_num_params(const pw_mlp *m) { return m ? (int64_t)m->nparam : 0; }

extern "C" int pw_mlp_get_params(const pw_mlp *m, float *host_out)
{
	if (!m || !host_out)
		return pw_fail(PW_ERR_INVALID_ARG, "pw_mlp_get_params: NULL argument");
	PW_CUDA(cudaSetDevice(m->device));
	PW_CUDA(cudaMemcpy(host_out, m->params.ptr, sizeof(float) * m->nparam, cudaMemcpyDeviceToHost));
	return PW_OK;
}

extern "C" int pw_mlp_set_params(pw_mlp *m, const float *host_in)
{
	if (!m || !host_in)
		return pw_fail(PW_ERR_INVALID_ARG, "pw_mlp_set_params: NULL argument");
	PW_CUDA(cudaSetDevice(m->device));
	PW_CUDA(cudaMemcpy(m->params.ptr, host_in, sizeof(float) * m->nparam, cudaMemcpyHostToDevice));
	m->wimg_dirty = true;
	for (int l = 0; l < NLAYER; l++) {
		const int64_t nw = (int64_t)H * in_dim(l);
		k_to_bf16<<<(unsigned)((nw + 255) / 256), 256>>>((float *)m->params.ptr + m->off_w[l], nw,
		                                                 (bf16 *)m->wbf.ptr + m->off_wb[l],
		                                                 (bf16 *)m->wbft.ptr + m->off_wb[l], H, in_dim(l));
	}
	PW_CUDA(cudaGetLastError());
	PW_CUDA(cudaDeviceSynchronize());
	return PW_OK;
}

extern "C" int pw_mlp_get_grads(const pw_mlp *m, float *host_out)
{
	if (!m || !host_out)
		return pw_fail(PW_ERR_INVALID_ARG, "pw_mlp_get_grads: NULL argument");
	PW_CUDA(cudaSetDevice(m->device));
	PW_CUDA(cudaMemcpy(host_out, m->grads.ptr, sizeof(float) * m->nparam, cudaMemcpyDeviceToHost));
	return PW_OK;
}

extern "C" int pw_mlp_get_adam(const pw_mlp *m, float *m1_out, float *m2_out, int64_t *step_out)
{
	if (!m)
		return pw_fail(PW_ERR_INVALID_ARG, "pw_mlp_get_adam: NULL network");
	PW_CUDA(cudaSetDevice(m->device));
	PW_CUDA(cudaDeviceSynchronize());
	if (m1_out)
		PW_CUDA(cudaMemcpy(m1_out, m->m1.ptr, sizeof(float) * m->nparam, cudaMemcpyDeviceToHost));
	if (m2_out)
		PW_CUDA(cudaMemcpy(m2_out, m->m2.ptr, sizeof(float) * m->nparam, cudaMemcpyDeviceToHost));
	if (step_out)
		*step_out = m->step;
	return PW_OK;
}

extern "C" int pw_mlp_set_adam(pw_mlp *m, const float *m1_in, const float *m2_in, int64_t step)
{
	if (!m)
		return pw_fail(PW_ERR_INVALID_ARG, "pw_mlp_set_adam: NULL network");
	if (step < 0)
		return pw_fail(PW_ERR_INVALID_ARG, "pw_mlp_set_adam: negative step count");
	PW_CUDA(cudaSetDevice(m->device));
	PW_CUDA(cudaDeviceSynchronize());
	if (m1_in)
		PW_CUDA(cudaMemcpy(m->m1.ptr, m1_in, sizeof(float) * m->nparam, cudaMemcpyHostToDevice));
	if (m2_in)
		PW_CUDA(cudaMemcpy(m->m2.ptr, m2_in, sizeof(float) * m->nparam, cudaMemcpyHostToDevice));
	m->step = step;
	return PW_OK;
}

static void launch_gemm_fwd(pw_mlp *m, int l, int64_t n, cudaStream_t st, bool keep_z)
{
	GemmArgs p;
	memset(&p, 0, sizeof(p));
	p.A = act(m, l);
	p.B = (const bf16 *)m->wbf.ptr + m->off_wb[l];
	p.M = (int)n;
	p.N = H;
	p.K = in_dim(l);
	p.lda = in_dim(l);
	p.ldb = in_dim(l);
	p.k_split = p.K;
	p.bias = (const float *)m->params.ptr + m->off_b[l];
	p.Zout = keep_z ? zbuf(m, l + 1) : nullptr;
	p.Y = act(m, l + 1);
	dim3 grid(H / BN, (unsigned)((n + BM - 1) / BM), 1);
	k_gemm<true, true, EPI_BIAS_SILU><<<grid, 256, 0, st>>>(p);
}

static int mlp_forward(pw_mlp *m, const double *states, int64_t n, cudaStream_t st, bool keep_z)
{
	k_features<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(states, n, act(m, 0));
	for (int l = 0; l < NLAYER; l++)
		launch_gemm_fwd(m, l, n, st, keep_z);
	PW_CUDA(cudaGetLastError());
	return PW_OK;
}

static int *mlp_err(pw_mlp *m) { return (int *)((char *)m->misc.ptr + 16); }

static int mlp_forward_tc(pw_mlp *m, const double *states, int64_t n, float *prob, int logits, void *stream);

// The weight-block schedule of a pair of tiles (see tc::Sched): the sequence of
// block uses, with stages chosen by Belady's rule (evict the content whose next
// use is farthest away); every content is released by its last use within the
// pair, so each pair starts with an empty ring.
static void build_schedule(int nslot, int &count, uint16_t *out)
{
	struct Use {
		int block, kb;
	};
	std::vector<Use> uses;
	for (int layer = 0; layer < NLAYER; layer++)
		for (int sl = 0; sl < nslot; sl++) {
			if (layer == 0) {
				uses.push_back({ 0, 0 });
				continue;
			}
			for (int u = 0; u < 4; u++) {
				const int j = sl == 0 ? u : 3 - u;
				uses.push_back({ 1 + 4 * (layer - 1) + j, j });
			}
		}
	const int U = (int)uses.size();
	std::vector<int> stage(U), load(U);
	int content[tc::NSTAGE] = { -1, -1, -1 }, last_used[tc::NSTAGE] = { -1, -1, -1 };
	auto next_use = [&](int block, int from) {
		for (int k = from; k < U; k++)
			if (uses[k].block == block)
				return k;
		return U + 1;
	};
	for (int i = 0; i < U; i++) {
		int s = -1;
		for (int t = 0; t < tc::NSTAGE; t++)
			if (content[t] == uses[i].block)
				s = t;
		load[i] = s < 0;
		if (s < 0) {
			// a stage whose content is dead, the least recently used first (so that loads
			// rotate through the ring and prefetch); else the farthest next use
			long best = -1;
			for (int t = 0; t < tc::NSTAGE; t++) {
				const int nu = content[t] < 0 ? U + 1 : next_use(content[t], i);
				const long key = nu > U ? 4L * U + (U - last_used[t]) : nu;
				if (key > best) {
					best = key;
					s = t;
				}
			}
			content[s] = uses[i].block;
		}
		stage[i] = s;
		last_used[s] = i;
	}
	for (int i = 0; i < U; i++) {
		// last use of this content: the next event on the stage is a load, or there is none
		bool last = true;
		for (int k = i + 1; k < U; k++)
			if (stage[k] == stage[i]) {
				last = load[k] != 0;
				break;
			}
		out[i] = (uint16_t)(uses[i].block | (stage[i] << 4) | (load[i] << 6) | ((last ? 1 : 0) << 7) |
		                    (uses[i].kb << 8));
	}
	count = U;
}

static float *mlp_head_table(pw_mlp *m)
{
	return (float *)((char *)m->wimg.ptr + (size_t)tc::NWBLOCK * tc::WBLOCK_BYTES);
}

extern "C" int pw_mlp_predict(pw_mlp *m, const double *states, int64_t n, float *prob, void *stream)
{
	PW_TRACE("pw_mlp_predict");
	return mlp_forward_tc(m, states, n, prob, 0, stream);
}

extern "C" int pw_mlp_score(pw_mlp *m, const double *states, int64_t n, float *logit, void *stream)
{
	PW_TRACE("pw_mlp_score");
	return mlp_forward_tc(m, states, n, logit, 1, stream);
}

// P(free) (or the logit) of n states on the tcgen05 tensor cores (one fused persistent kernel).
static int mlp_forward_tc(pw_mlp *m, const double *states, int64_t n, float *prob, int logits, void *stream)
{
	if (!m || n < 0 || (n > 0 && (!states || !prob)))
		return pw_fail(PW_ERR_INVALID_ARG, logits ? "pw_mlp_score: bad argument" : "pw_mlp_predict: bad argument");
	if (n == 0)
		return PW_OK;
	PW_CUDA(cudaSetDevice(m->device));
	cudaStream_t st = (cudaStream_t)stream;
	if (m->wimg_dirty) {
		PW_CUDA(m->wimg.reserve((size_t)tc::NWBLOCK * tc::WBLOCK_BYTES + sizeof(float) * tc::HT_FLOATS));
		const int64_t nchunk = (int64_t)tc::NWBLOCK * H * 8;
		tc::k_weight_image<<<(unsigned)((nchunk + 255) / 256), 256, 0, st>>>(
		    (const float *)m->params.ptr, (int64_t)m->off_w[0], (int64_t)m->off_w[1], (int64_t)m->off_w[2],
		    (int64_t)m->off_w[3], (bf16 *)m->wimg.ptr);
		tc::k_head_table<<<(tc::HT_FLOATS + 255) / 256, 256, 0, st>>>(
		    (const float *)m->params.ptr, (int64_t)m->off_b[0], (int64_t)m->off_b[1], (int64_t)m->off_b[2],
		    (int64_t)m->off_b[3], (int64_t)m->off_w5, (int64_t)m->off_b5, mlp_head_table(m));
		PW_CUDA(cudaGetLastError());
		// the epilogue reads its constants from the launch's parameter bank (warp-uniform
		// operands), so keep a host copy: one small synchronous copy per weight update
		m->ht_host.resize(tc::HT_FLOATS);
		PW_CUDA(cudaMemcpyAsync(m->ht_host.data(), mlp_head_table(m), sizeof(float) * tc::HT_FLOATS,
		                        cudaMemcpyDeviceToHost, st));
		PW_CUDA(cudaStreamSynchronize(st));
		m->wimg_dirty = false;
	}
	static bool attr_set = false;
	if (!attr_set) {
		PW_CUDA(cudaFuncSetAttribute(tc::k_mlp_forward_tc, cudaFuncAttributeMaxDynamicSharedMemorySize,
		                             tc::SMEM_BYTES));
		attr_set = true;
	}
	tc::FwdArgs a;
	memset(&a, 0, sizeof(a));
	build_schedule(1, a.sched.n[0], a.sched.e[0]);
	build_schedule(2, a.sched.n[1], a.sched.e[1]);
	a.states = states;
	a.n = n;
	a.wimg = (const bf16 *)m->wimg.ptr;
	memcpy(a.ht, m->ht_host.data(), sizeof(a.ht));
	a.prob = prob;
	a.logits = logits;
	a.withhold = m->withhold_next ? 1 : 0;
	m->withhold_next = false;
	a.err = mlp_err(m);
	const int64_t ntiles = (n + tc::TILE_M - 1) / tc::TILE_M;
	const unsigned grid = (unsigned)std::min<int64_t>(ntiles, m->num_sms);
	tc::k_mlp_forward_tc<<<grid, tc::NTHREADS, tc::SMEM_BYTES, st>>>(a);
	PW_CUDA(cudaGetLastError());
	return PW_OK;
}

extern "C" int pw_select_top(const float *score, const double *states, int64_t n, int64_t k, double *out_states,
                             int64_t capacity, int64_t *out_count, void *stream)
{
	PW_TRACE("pw_select_top");
	if (n < 0 || k < 0 || capacity < 0 || !out_count || (n > 0 && (!score || !states)) ||
	    (capacity > 0 && !out_states))
		return pw_fail(PW_ERR_INVALID_ARG, "pw_select_top: bad argument");
	*out_count = 0;
	if (n == 0 || k == 0)
		return PW_OK;
	k = std::min(k, n);
	cudaStream_t st = (cudaStream_t)stream;
	int dev = 0, sms = 1;
	PW_CUDA(cudaGetDevice(&dev));
	PW_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
	DeviceBuffer hist;
	PW_CUDA(hist.reserve(sizeof(unsigned long long) * (2048 + 1)));
	unsigned long long *dh = (unsigned long long *)hist.ptr;
	std::vector<unsigned long long> h(2048);
	const unsigned grid = (unsigned)std::min<int64_t>((n + 255) / 256, (int64_t)sms * 8);
	uint32_t prefix = 0;   // bits of the k-th largest score found so far
	int64_t above = 0;     // scores strictly above the current prefix range
	for (int pass = 0; pass < 3; pass++) {
		const int nb = 1 << SEL_BITS[pass];
		const int pshift = SEL_SHIFT[pass] + SEL_BITS[pass];   // bits above this pass
		PW_CUDA(cudaMemsetAsync(dh, 0, sizeof(unsigned long long) * nb, st));
		k_score_hist<<<grid, 256, 0, st>>>(score, n, SEL_SHIFT[pass], SEL_BITS[pass], prefix, pass == 0 ? 32 : pshift,
		                                   dh);
		PW_CUDA(cudaGetLastError());
		PW_CUDA(cudaMemcpyAsync(h.data(), dh, sizeof(unsigned long long) * nb, cudaMemcpyDeviceToHost, st));
		PW_CUDA(cudaStreamSynchronize(st));
		int b = nb - 1;
		for (; b > 0; b--) {
			if (above + (int64_t)h[b] >= k)
				break;
			above += (int64_t)h[b];
		}
		prefix = (prefix << SEL_BITS[pass]) | (uint32_t)b;
	}
	const uint32_t thr = prefix;
	unsigned long long *dc = dh + 2048;
	PW_CUDA(cudaMemsetAsync(dc, 0, sizeof(unsigned long long), st));
	k_select_states<<<grid, 256, 0, st>>>(score, states, n, thr, out_states, capacity, dc);
	PW_CUDA(cudaGetLastError());
	unsigned long long cnt = 0;
	PW_CUDA(cudaMemcpyAsync(&cnt, dc, sizeof(cnt), cudaMemcpyDeviceToHost, st));
	PW_CUDA(cudaStreamSynchronize(st));
	*out_count = (int64_t)cnt;
	if ((int64_t)cnt > capacity)
		return pw_fail(PW_ERR_CAPACITY, "pw_select_top: " + std::to_string(cnt) + " states tie at or above the "
		                                    "k-th score; capacity " + std::to_string(capacity));
	return PW_OK;
}

extern "C" int pw_mlp_check(pw_mlp *m)
{
	if (!m)
		return pw_fail(PW_ERR_INVALID_ARG, "pw_mlp_check: NULL network");
	PW_CUDA(cudaSetDevice(m->device));
	PW_CUDA(cudaDeviceSynchronize());
	int err = 0;
	PW_CUDA(cudaMemcpy(&err, mlp_err(m), sizeof(int), cudaMemcpyDeviceToHost));
	if (err) {
		PW_CUDA(cudaMemset(mlp_err(m), 0, sizeof(int)));
		return pw_fail(PW_ERR_INTERNAL, "pw_mlp: a device wait of the tcgen05 forward kernel gave up (site " +
		                                    std::to_string(err) + ")");
	}
	return PW_OK;
}

// The same network through the mma.sync GEMM kernels that training uses.
extern "C" int pw_mlp_withhold_next_weights(pw_mlp *m)
{
	if (!m)
		return pw_fail(PW_ERR_INVALID_ARG, "pw_mlp_withhold_next_weights: NULL network");
	m->withhold_next = true;
	return PW_OK;
}

extern "C" int pw_mlp_predict_mma(pw_mlp *m, const double *states, int64_t n, float *prob, void *stream)
{
	PW_TRACE("pw_mlp_predict_mma");
	if (!m || n < 0 || (n > 0 && (!states || !prob)))
		return pw_fail(PW_ERR_INVALID_ARG, "pw_mlp_predict_mma: bad argument");
	if (n == 0)
		return PW_OK;
	PW_CUDA(cudaSetDevice(m->device));
	cudaStream_t st = (cudaStream_t)stream;
	const int64_t chunk = int64_t(1) << 22;
	int rc = mlp_reserve(m, std::min(n, chunk));
	if (rc)
		return rc;
	for (int64_t s0 = 0; s0 < n; s0 += chunk) {
		const int64_t c = std::min(chunk, n - s0);
		rc = mlp_forward(m, states + 7 * s0, c, st, false);
		if (rc)
			return rc;
		k_head_forward<<<(unsigned)((c * 32 + 255) / 256), 256, 0, st>>>(
		    act(m, NLAYER), (const float *)m->params.ptr + m->off_w5, (const float *)m->params.ptr + m->off_b5, c,
		    nullptr, prob + s0);
	}
	PW_CUDA(cudaGetLastError());
	return PW_OK;
}

// Gradients of the mean binary cross-entropy of one batch into the grads block
// (no update); *loss_out gets the loss (synchronises the stream).
// ------------------------------------------------------------------ tcgen05 training step

typedef PFN_cuTensorMapEncodeTiled_v12000 EncodeFn;

static EncodeFn encode_fn()
{
	static EncodeFn fn = nullptr;
	if (!fn) {
		void *p = nullptr;
		cudaDriverEntryPointQueryResult q;
		if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
		        cudaSuccess &&
		    q == cudaDriverEntryPointSuccess)
			fn = (EncodeFn)p;
	}
	return fn;
}

// Tensor map of a row-major BF16 matrix [rows][cols] with row pitch `ld` elements,
// box = 64 columns x box_rows rows, 128-byte swizzle.
static int make_map(CUtensorMap *map, const bf16 *base, int64_t rows, int64_t cols, int64_t ld, int box_rows)
{
	EncodeFn enc = encode_fn();
	if (!enc)
		return pw_fail(PW_ERR_CUDA, "cuTensorMapEncodeTiled is not available from the driver");
	if (((uintptr_t)base & 15) || ((ld * 2) & 15))
		return pw_fail(PW_ERR_INTERNAL, "tensor map: base or row pitch not 16-byte aligned");
	const cuuint64_t dims[2] = { (cuuint64_t)cols, (cuuint64_t)rows };
	const cuuint64_t strides[1] = { (cuuint64_t)(ld * 2) };
	const cuuint32_t box[2] = { 64u, (cuuint32_t)box_rows };
	const cuuint32_t estr[2] = { 1u, 1u };
	const CUresult r = enc(map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, (void *)base, dims, strides, box, estr,
	                       CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
	                       CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
	if (r != CUDA_SUCCESS)
		return pw_fail(PW_ERR_CUDA, "cuTensorMapEncodeTiled failed (" + std::to_string((int)r) + ")");
	return PW_OK;
}

template <int NT, int EPI, int STAGES>
static int run_gemm(const CUtensorMap &ta, const CUtensorMap &tb, const tt::Args &a, int splits, cudaStream_t st)
{
	typedef tt::Cfg<NT, STAGES> C;
	static bool attr = false;
	if (!attr) {
		PW_CUDA(cudaFuncSetAttribute(tt::k_gemm_tc<NT, EPI, STAGES>, cudaFuncAttributeMaxDynamicSharedMemorySize,
		                             C::SMEM));
		attr = true;
	}
	dim3 grid((unsigned)((a.M + tt::BM - 1) / tt::BM), (unsigned)((a.N + NT - 1) / NT), (unsigned)splits);
	tt::k_gemm_tc<NT, EPI, STAGES><<<grid, tt::NTHREADS, C::SMEM, st>>>(ta, tb, a);
	PW_CUDA(cudaGetLastError());
	return PW_OK;
}

// Bias gradient: column sums of G [n][256].
static void colsum(const bf16 *G, int64_t n, float *out, int num_sms, cudaStream_t st)
{
	const int64_t blocks = std::max<int64_t>(1, std::min<int64_t>((n + 255) / 256, (int64_t)num_sms * 4));
	const int64_t rows = (n + blocks - 1) / blocks;
	tt::k_colsum_v<<<(unsigned)blocks, 256, 0, st>>>(G, n, rows, out);
}

static int tc_reserve(pw_mlp *m, int64_t rows)
{
	if (rows <= m->tcap)
		return PW_OK;
	const int64_t r = ((rows + 127) / 128) * 128;
	PW_CUDA(m->x64.reserve(sizeof(bf16) * (size_t)r * 64));
	PW_CUDA(m->xt.reserve(sizeof(bf16) * (size_t)r * KIN));
	PW_CUDA(m->ht.reserve(sizeof(bf16) * (size_t)r * H * 3));    // H1t, H2t, H3t
	PW_CUDA(m->gt.reserve(sizeof(bf16) * (size_t)r * H));
	m->tcap = r;
	return PW_OK;
}

static int mlp_backward_tc(pw_mlp *m, const double *states, const uint8_t *labels, int64_t n, cudaStream_t st,
                           float *loss_out)
{
	int rc = mlp_reserve(m, n);
	if (rc || (rc = tc_reserve(m, n)))
		return rc;
	const int64_t ldt = m->tcap;
	float *P = (float *)m->params.ptr, *G = (float *)m->grads.ptr;
	float *logit = (float *)m->head.ptr, *gs = logit + m->cap;
	float *loss = (float *)m->misc.ptr;
	int *err = mlp_err(m);
	bf16 *x64 = (bf16 *)m->x64.ptr, *xt = (bf16 *)m->xt.ptr, *ht = (bf16 *)m->ht.ptr, *gt = (bf16 *)m->gt.ptr;
	auto Ht = [&](int l) { return ht + (size_t)(l - 1) * H * ldt; };   // H_l^T, l = 1..3
	PW_CUDA(m->w1p.reserve(sizeof(bf16) * H * 64));
	k_w1_pad<<<(H * 64 + 255) / 256, 256, 0, st>>>(P + m->off_w[0], (bf16 *)m->w1p.ptr);
	k_features64<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(states, n, x64, xt, ldt);
	PW_CUDA(cudaGetLastError());
	// forward: Z_{l+1}, H_{l+1} (row-major), H_{l+1}^T
	for (int l = 0; l < NLAYER; l++) {
		CUtensorMap ta, tb;
		const int K = l == 0 ? 64 : H;
		const bf16 *A = l == 0 ? x64 : act(m, l);
		const bf16 *B = l == 0 ? (const bf16 *)m->w1p.ptr : (const bf16 *)m->wbf.ptr + m->off_wb[l];
		if ((rc = make_map(&ta, A, n, K, K, tt::BM)) || (rc = make_map(&tb, B, H, K, K, 256)))
			return rc;
		tt::Args a;
		memset(&a, 0, sizeof(a));
		a.M = (int)n;
		a.N = H;
		a.K = K;
		a.k_split = K;
		a.bias = P + m->off_b[l];
		a.Z = zbuf(m, l + 1);
		a.Y = act(m, l + 1);
		a.Yt = l + 1 < NLAYER ? Ht(l + 1) : nullptr;
		a.ldt = ldt;
		a.err = err;
		if ((rc = run_gemm<256, tt::E_FWD, 2>(ta, tb, a, 1, st)))
			return rc;
	}
	PW_CUDA(cudaMemsetAsync(G, 0, sizeof(float) * m->nparam, st));
	PW_CUDA(cudaMemsetAsync(loss, 0, sizeof(float), st));
	k_head_forward<<<(unsigned)((n * 32 + 255) / 256), 256, 0, st>>>(act(m, NLAYER), P + m->off_w5, P + m->off_b5, n,
	                                                                  logit, nullptr);
	k_head_loss<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(logit, labels, n, gs, loss);
	bf16 *Gcur = (bf16 *)m->gbuf.ptr, *Gnext = (bf16 *)m->gbuf2.ptr;
	tt::k_head_backward_t<<<(unsigned)std::min<int64_t>((n + 63) / 64, (int64_t)m->num_sms * 8), 256, 0, st>>>(
	    act(m, NLAYER), zbuf(m, NLAYER), gs, P + m->off_w5, n, G + m->off_w5, G + m->off_b5, Gcur, gt, ldt);
	PW_CUDA(cudaGetLastError());
	// split the batch so that the weight-gradient GEMMs fill the GPU (2 M tiles each)
	const int64_t kblocks = (n + 63) / 64;
	const int64_t splits = std::max<int64_t>(1, std::min<int64_t>(kblocks, (int64_t)m->num_sms / 2));
	const int k_split = (int)(((kblocks + splits - 1) / splits) * 64);
	const int nsplit = (int)((n + k_split - 1) / k_split);
	PW_CUDA(m->dw_ws.reserve(sizeof(float) * (size_t)nsplit * H * H));
	for (int l = NLAYER - 1; l >= 0; l--) {
		// dW_l = G^T X_l: A = G^T [256][n], B = X_l^T [in][n], K = batch
		const int in = l == 0 ? KIN : H;
		CUtensorMap ta, tb;
		if ((rc = make_map(&ta, gt, H, n, ldt, tt::BM)) ||
		    (rc = make_map(&tb, l == 0 ? xt : Ht(l), in, n, ldt, in == H ? 256 : 16)))
			return rc;
		tt::Args a;
		memset(&a, 0, sizeof(a));
		a.M = H;
		a.N = in;
		a.K = (int)n;
		a.k_split = k_split;
		a.C = (float *)m->dw_ws.ptr;
		a.err = err;
		if ((rc = in == H ? run_gemm<256, tt::E_DW, 4>(ta, tb, a, nsplit, st)
		                  : run_gemm<16, tt::E_DW, 4>(ta, tb, a, nsplit, st)))
			return rc;
		const int64_t cnt = (int64_t)H * in;
		tt::k_reduce_splits<<<(unsigned)((cnt + 255) / 256), 256, 0, st>>>((const float *)m->dw_ws.ptr, nsplit, cnt,
		                                                                  G + m->off_w[l]);
		colsum(Gcur, n, G + m->off_b[l], m->num_sms, st);
		PW_CUDA(cudaGetLastError());
		if (l == 0)
			break;
		// G_l = (G W_l) * SiLU'(Z_l): A = G [n][256], B = W_l^T [in][out]
		if ((rc = make_map(&ta, Gcur, n, H, H, tt::BM)) ||
		    (rc = make_map(&tb, (const bf16 *)m->wbft.ptr + m->off_wb[l], H, H, H, 256)))
			return rc;
		memset(&a, 0, sizeof(a));
		a.M = (int)n;
		a.N = H;
		a.K = H;
		a.k_split = H;
		a.Z = zbuf(m, l);
		a.Y = Gnext;
		a.Yt = gt;
		a.ldt = ldt;
		a.err = err;
		if ((rc = run_gemm<256, tt::E_DX, 2>(ta, tb, a, 1, st)))
			return rc;
		bf16 *t = Gcur;
		Gcur = Gnext;
		Gnext = t;
	}
	if (loss_out) {
		PW_CUDA(cudaMemcpyAsync(loss_out, loss, sizeof(float), cudaMemcpyDeviceToHost, st));
		PW_CUDA(cudaStreamSynchronize(st));
	}
	return PW_OK;
}

static int mlp_backward(pw_mlp *m, const double *states, const uint8_t *labels, int64_t n, cudaStream_t st,
                        float *loss_out)
{
	if (!m->mma_training)
		return mlp_backward_tc(m, states, labels, n, st, loss_out);
	int rc = mlp_reserve(m, n);
	if (rc)
		return rc;
	rc = mlp_forward(m, states, n, st, true);
	if (rc)
		return rc;
	float *P = (float *)m->params.ptr, *G = (float *)m->grads.ptr;
	float *logit = (float *)m->head.ptr, *gs = logit + m->cap;
	float *loss = (float *)m->misc.ptr;
	PW_CUDA(cudaMemsetAsync(G, 0, sizeof(float) * m->nparam, st));
	PW_CUDA(cudaMemsetAsync(loss, 0, sizeof(float), st));
	k_head_forward<<<(unsigned)((n * 32 + 255) / 256), 256, 0, st>>>(act(m, NLAYER), P + m->off_w5, P + m->off_b5, n,
	                                                                  logit, nullptr);
	k_head_loss<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(logit, labels, n, gs, loss);
	bf16 *Gcur = (bf16 *)m->gbuf.ptr, *Gnext = (bf16 *)m->gbuf2.ptr;
	k_head_backward<<<304, 256, 0, st>>>(act(m, NLAYER), zbuf(m, NLAYER), gs, P + m->off_w5, n, G + m->off_w5,
	                                     G + m->off_b5, Gcur);
	for (int l = NLAYER - 1; l >= 0; l--) {
		// Gcur = dL/dZ_{l+1} [n x H]
		// dW_l [H x in] += Gcur^T X_l  (split over the batch)
		GemmArgs p;
		memset(&p, 0, sizeof(p));
		p.A = Gcur;               // A(m = out, k = row): stored [row][out] -> not k-contiguous
		p.B = act(m, l);          // B(n = in, k = row): stored [row][in] -> not k-contiguous
		p.M = H;
		p.N = in_dim(l);
		p.K = (int)n;
		p.lda = H;
		p.ldb = in_dim(l);
		p.k_split = 2048;
		p.Cf = G + m->off_w[l];
		dim3 grid((unsigned)((in_dim(l) + BN - 1) / BN), H / BM, (unsigned)((n + p.k_split - 1) / p.k_split));
		if (in_dim(l) == KIN)
			k_gemm<false, false, EPI_ATOMIC_F32><<<grid, 256, 0, st>>>(p);
		else
			k_gemm<false, false, EPI_ATOMIC_F32><<<grid, 256, 0, st>>>(p);
		k_colsum<<<256, H, 0, st>>>(Gcur, n, G + m->off_b[l]);
		if (l == 0)
			break;
		// dL/dZ_l = (Gcur W_l) * SiLU'(Z_l)
		GemmArgs q;
		memset(&q, 0, sizeof(q));
		q.A = Gcur;                                          // [row][out], k = out contiguous
		q.B = (const bf16 *)m->wbft.ptr + m->off_wb[l];      // W^T [in][out], k = out contiguous
		q.M = (int)n;
		q.N = H;
		q.K = H;
		q.lda = H;
		q.ldb = H;
		q.k_split = H;
		q.Zin = zbuf(m, l);
		q.Y = Gnext;
		dim3 g2(H / BN, (unsigned)((n + BM - 1) / BM), 1);
		k_gemm<true, true, EPI_DSILU><<<g2, 256, 0, st>>>(q);
		bf16 *t = Gcur;
		Gcur = Gnext;
		Gnext = t;
	}
	PW_CUDA(cudaGetLastError());
	if (loss_out) {
		PW_CUDA(cudaMemcpyAsync(loss_out, loss, sizeof(float), cudaMemcpyDeviceToHost, st));
		PW_CUDA(cudaStreamSynchronize(st));
	}
	return PW_OK;
}

extern "C" int pw_mlp_gradients(pw_mlp *m, const double *states, const uint8_t *labels, int64_t n, float *loss_out,
                                void *stream)
{
	PW_TRACE("pw_mlp_gradients");
	if (!m || n <= 0 || !states || !labels)
		return pw_fail(PW_ERR_INVALID_ARG, "pw_mlp_gradients: bad argument");
	if (n > (int64_t(1) << 24))
		return pw_fail(PW_ERR_INVALID_ARG, "pw_mlp_gradients: at most 2^24 rows per batch");
	PW_CUDA(cudaSetDevice(m->device));
	return mlp_backward(m, states, labels, n, (cudaStream_t)stream, loss_out);
}

// One Adam step on a batch (device states and 0/1 labels, 1 = free).
extern "C" int pw_mlp_set_training_kernels(pw_mlp *m, int use_mma)
{
	if (!m)
		return pw_fail(PW_ERR_INVALID_ARG, "pw_mlp_set_training_kernels: NULL network");
	m->mma_training = use_mma != 0;
	return PW_OK;
}

extern "C" int pw_mlp_train_step(pw_mlp *m, const double *states, const uint8_t *labels, int64_t n, float lr,
                                 float *loss_out, void *stream)
{
	PW_TRACE("pw_mlp_train_step");
	int rc = pw_mlp_gradients(m, states, labels, n, loss_out, stream);
	if (rc)
		return rc;
	cudaStream_t st = (cudaStream_t)stream;
	m->step++;
	m->wimg_dirty = true;
	const float c1 = 1.f - std::pow(m->b1, (float)m->step), c2 = 1.f - std::pow(m->b2, (float)m->step);
	float *P = (float *)m->params.ptr, *G = (float *)m->grads.ptr, *M1 = (float *)m->m1.ptr, *M2 = (float *)m->m2.ptr;
	for (int l = 0; l < NLAYER; l++) {
		const int64_t nw = (int64_t)H * in_dim(l);
		k_adam<<<(unsigned)((nw + 255) / 256), 256, 0, st>>>(P + m->off_w[l], G + m->off_w[l], M1 + m->off_w[l],
		                                                     M2 + m->off_w[l], nw, lr, m->b1, m->b2, m->eps, c1, c2,
		                                                     (bf16 *)m->wbf.ptr + m->off_wb[l],
		                                                     (bf16 *)m->wbft.ptr + m->off_wb[l], H, in_dim(l));
		k_adam<<<1, H, 0, st>>>(P + m->off_b[l], G + m->off_b[l], M1 + m->off_b[l], M2 + m->off_b[l], H, lr, m->b1,
		                        m->b2, m->eps, c1, c2, nullptr, nullptr, 1, H);
	}
	k_adam<<<1, H + 1, 0, st>>>(P + m->off_w5, G + m->off_w5, M1 + m->off_w5, M2 + m->off_w5, H + 1, lr, m->b1, m->b2,
	                            m->eps, c1, c2, nullptr, nullptr, 1, H + 1);
	PW_CUDA(cudaGetLastError());
	return PW_OK;
}
