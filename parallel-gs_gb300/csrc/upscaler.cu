// Learned anti-aliasing upscaler: 6 conv layers, 3x3, 32 channels, ReLU,
// residual over the input image.  BF16 activations and weights, FP32
// accumulation on the tensor cores; FP32 master weights trained with Adam.
//
// Layout: activations NHWC in BF16 with 16 (input, last-layer gradient) or 32
// channels.  A convolution is an implicit GEMM: M = pixels of a 16x16 tile,
// N = output channels, K = 9 taps x input channels.  Each CTA stages the
// 18x18 input halo and the layer's weights in shared memory; each warp owns
// two 16-pixel rows and all output channels.
//
//   layer 0: 4 (padded to 16) -> 32, ReLU
//   layers 1-4: 32 -> 32, ReLU
//   layer 5: 32 -> 4 (padded to 8), output = input + conv
//
// The same kernel computes the data gradient (flipped, transposed weights;
// the epilogue multiplies by the ReLU mask of the layer below), and a second
// kernel the weight gradient (K = pixels).
#include "pgs.h"
#include "umma.cuh"

#include <cuda.h>
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <new>
#include <utility>
#include <vector>

namespace pgs_up
{
constexpr int LAYERS = 6;
constexpr int TILE = 16;
constexpr int HALO = TILE + 2;
constexpr int REAL_IN[LAYERS] = { 4, 32, 32, 32, 32, 32 };
constexpr int REAL_OUT[LAYERS] = { 32, 32, 32, 32, 32, 4 };
constexpr int PAD_IN[LAYERS] = { 16, 32, 32, 32, 32, 32 };
constexpr int PAD_OUT[LAYERS] = { 32, 32, 32, 32, 32, 8 };
// Device copies of the layer shapes.
__constant__ int d_real_in[LAYERS] = { 4, 32, 32, 32, 32, 32 };
__constant__ int d_real_out[LAYERS] = { 32, 32, 32, 32, 32, 4 };
__constant__ int d_pad_in[LAYERS] = { 16, 32, 32, 32, 32, 32 };
__constant__ int d_pad_out[LAYERS] = { 32, 32, 32, 32, 32, 8 };

#define UP_TRY(x)                                                                                                      \
	do                                                                                                                 \
	{                                                                                                                  \
		cudaError_t e_ = (x);                                                                                          \
		if (e_ != cudaSuccess)                                                                                         \
			return PGS_ERROR_CUDA;                                                                                     \
	} while (0)

__device__ __forceinline__ uint32_t smem_u32(const void *p) { return uint32_t(__cvta_generic_to_shared(p)); }

__device__ __forceinline__ void ldsm_x4(uint32_t addr, uint32_t &r0, uint32_t &r1, uint32_t &r2, uint32_t &r3)
{
	asm volatile("ldmatrix.sync.aligned.m8n8.x4.shared.b16 {%0,%1,%2,%3}, [%4];\n"
	             : "=r"(r0), "=r"(r1), "=r"(r2), "=r"(r3) : "r"(addr));
}

__device__ __forceinline__ void ldsm_x4_t(uint32_t addr, uint32_t &r0, uint32_t &r1, uint32_t &r2, uint32_t &r3)
{
	asm volatile("ldmatrix.sync.aligned.m8n8.x4.trans.shared.b16 {%0,%1,%2,%3}, [%4];\n"
	             : "=r"(r0), "=r"(r1), "=r"(r2), "=r"(r3) : "r"(addr));
}

__device__ __forceinline__ void ldsm_x2(uint32_t addr, uint32_t &r0, uint32_t &r1)
{
	asm volatile("ldmatrix.sync.aligned.m8n8.x2.shared.b16 {%0,%1}, [%2];\n" : "=r"(r0), "=r"(r1) : "r"(addr));
}

__device__ __forceinline__ void ldsm_x2_t(uint32_t addr, uint32_t &r0, uint32_t &r1)
{
	asm volatile("ldmatrix.sync.aligned.m8n8.x2.trans.shared.b16 {%0,%1}, [%2];\n" : "=r"(r0), "=r"(r1) : "r"(addr));
}

// D = A(16x16, row) * B(16x8, col) + D, BF16 in, FP32 accumulate.
__device__ __forceinline__ void mma_bf16(float *d, const uint32_t *a, uint32_t b0, uint32_t b1)
{
	asm volatile("mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
	             "{%0,%1,%2,%3};\n"
	             : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
	             : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

__device__ __forceinline__ uint32_t pack_bf16x2(float lo, float hi)
{
	__nv_bfloat162 v = __floats2bfloat162_rn(lo, hi);
	return *reinterpret_cast<uint32_t *>(&v);
}

// One RGBA8 pixel as the network's first four input channels (x / 255 in
// BF16), two channels per word.
__device__ __forceinline__ void rgba8_to_bf16x4(uint32_t c, uint32_t &rg, uint32_t &ba)
{
	rg = pack_bf16x2(float(c & 0xffu) / 255.0f, float((c >> 8) & 0xffu) / 255.0f);
	ba = pack_bf16x2(float((c >> 16) & 0xffu) / 255.0f, float(c >> 24) / 255.0f);
}

// Programmatic dependent launch.  launch_dependents lets the next kernel of
// the stream start its CTAs (their set-up) once every CTA of this one has
// started; wait blocks until every kernel this one depends on has finished
// and its writes are visible.  Both do nothing when the launch did not ask
// for it.
__device__ __forceinline__ void griddep_launch_dependents()
{
	asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
}

__device__ __forceinline__ void griddep_wait()
{
	asm volatile("griddepcontrol.wait;" ::: "memory");
}

// Epilogue kinds of conv3x3_kernel.
enum : int
{
	EPI_RELU = 0,   // out = bf16(relu(acc + bias))
	EPI_LAST = 1,   // out_f32 = acc + bias + input image; optional RGBA8 copy
	EPI_MASK = 2,   // out = bf16(acc * (mask > 0))  (data gradient through ReLU)
};

struct ConvArgs
{
	const __nv_bfloat16 *in;     // N x H x W x CIN
	const uint8_t *in_rgba;      // CIN 16 only: N x H x W x 4 RGBA8 read in place of `in` (converted as by image_to_bf16_kernel)
	const __nv_bfloat16 *wt;     // 9 x COUT x CIN (tap, out channel, in channel)
	const float *bias;           // COUT (EPI_RELU / EPI_LAST)
	__nv_bfloat16 *out;          // N x H x W x COUT (EPI_RELU / EPI_MASK)
	const __nv_bfloat16 *mask;   // N x H x W x COUT (EPI_MASK)
	const uint8_t *image;        // N x H x W x 4 RGBA8 input image (EPI_LAST)
	float *out_f32;              // N x H x W x 4 (EPI_LAST)
	uint8_t *out_rgba;           // N x H x W x 4 (EPI_LAST, optional)
	int n, h, w;
};

// Grid: (ceil(W/16), ceil(H/16), N); 256 threads.
template <int CIN, int COUT, int EPI>
__global__ void __launch_bounds__(256) conv3x3_kernel(ConvArgs A)
{
	constexpr int PS = CIN + 8;        // padded pixel stride (elements): conflict-free ldmatrix rows
	constexpr int NT = COUT / 8;       // n8 tiles
	__shared__ __align__(16) __nv_bfloat16 s_in[HALO * HALO * PS];
	__shared__ __align__(16) __nv_bfloat16 s_w[9 * COUT * PS];

	const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
	const int x0 = blockIdx.x * TILE, y0 = blockIdx.y * TILE, img = blockIdx.z;
	griddep_launch_dependents();

	// Weights (not written by the kernels before this one), then the wait
	// for the previous layer, then its output.
	constexpr int CH = CIN / 8;
	for (int i = tid; i < 9 * COUT * CH; i += 256)
	{
		int r = i / CH, c = (i % CH) * 8;
		*reinterpret_cast<uint4 *>(s_w + r * PS + c) = *reinterpret_cast<const uint4 *>(A.wt + r * CIN + c);
	}
	griddep_wait();

	// Input halo, 16-byte chunks, zero outside the image.
	if (CIN == 16 && A.in_rgba)
	{
		// The RGBA8 image itself: channels 0-3 scaled by 1/255, 4-15 zero.
		for (int p = tid; p < HALO * HALO; p += 256)
		{
			int gx = x0 - 1 + p % HALO, gy = y0 - 1 + p / HALO;
			uint4 v = make_uint4(0, 0, 0, 0);
			if (gx >= 0 && gy >= 0 && gx < A.w && gy < A.h)
			{
				const uint32_t c = reinterpret_cast<const uint32_t *>(A.in_rgba)[(size_t(img) * A.h + gy) * A.w + gx];
				rgba8_to_bf16x4(c, v.x, v.y);
			}
			*reinterpret_cast<uint4 *>(s_in + p * PS) = v;
			*reinterpret_cast<uint4 *>(s_in + p * PS + 8) = make_uint4(0, 0, 0, 0);
		}
	}
	else
	for (int i = tid; i < HALO * HALO * CH; i += 256)
	{
		int p = i / CH, c = (i % CH) * 8;
		int gx = x0 - 1 + p % HALO, gy = y0 - 1 + p / HALO;
		uint4 v = make_uint4(0, 0, 0, 0);
		if (gx >= 0 && gy >= 0 && gx < A.w && gy < A.h)
			v = *reinterpret_cast<const uint4 *>(A.in + ((size_t(img) * A.h + gy) * A.w + gx) * CIN + c);
		*reinterpret_cast<uint4 *>(s_in + p * PS + c) = v;
	}
	__syncthreads();

	float acc[2][NT][4];
	#pragma unroll
	for (int r = 0; r < 2; r++)
		#pragma unroll
		for (int j = 0; j < NT; j++)
			#pragma unroll
			for (int k = 0; k < 4; k++)
				acc[r][j][k] = 0.0f;

	#pragma unroll 1
	for (int tap = 0; tap < 9; tap++)
	{
		const int dy = tap / 3, dx = tap % 3;
		#pragma unroll
		for (int kc = 0; kc < CIN / 16; kc++)
		{
			uint32_t a[2][4];
			#pragma unroll
			for (int r = 0; r < 2; r++)
			{
				int py = warp * 2 + r + dy, px = (lane & 15) + dx;
				const __nv_bfloat16 *p = s_in + (py * HALO + px) * PS + kc * 16 + (lane >> 4) * 8;
				ldsm_x4(smem_u32(p), a[r][0], a[r][1], a[r][2], a[r][3]);
			}
			#pragma unroll
			for (int j = 0; j < NT; j += 2)
			{
				if (j + 1 < NT)
				{
					// Two n-tiles: lanes 0-15 tile j (k 0-7, 8-15), 16-31 tile j+1.
					int nt = j + (lane >> 4), nrow = nt * 8 + (lane & 7), kh = (lane >> 3) & 1;
					const __nv_bfloat16 *p = s_w + (tap * COUT + nrow) * PS + kc * 16 + kh * 8;
					uint32_t b0, b1, b2, b3;
					ldsm_x4(smem_u32(p), b0, b1, b2, b3);
					#pragma unroll
					for (int r = 0; r < 2; r++)
					{
						mma_bf16(acc[r][j], a[r], b0, b1);
						mma_bf16(acc[r][j + 1], a[r], b2, b3);
					}
				}
				else
				{
					int nrow = j * 8 + (lane & 7), kh = (lane >> 3) & 1;
					const __nv_bfloat16 *p = s_w + (tap * COUT + nrow) * PS + kc * 16 + kh * 8;
					uint32_t b0, b1;
					ldsm_x2(smem_u32(p), b0, b1);
					#pragma unroll
					for (int r = 0; r < 2; r++)
						mma_bf16(acc[r][j], a[r], b0, b1);
				}
			}
		}
	}

	// Epilogue: thread holds rows g, g+8 and columns 2t, 2t+1 of each tile.
	const int g = lane >> 2, t = lane & 3;
	#pragma unroll
	for (int r = 0; r < 2; r++)
	{
		const int gy = y0 + warp * 2 + r;
		#pragma unroll
		for (int half = 0; half < 2; half++)
		{
			const int gx = x0 + g + half * 8;
			if (gx >= A.w || gy >= A.h)
				continue;
			const size_t pix = (size_t(img) * A.h + gy) * A.w + gx;
			#pragma unroll
			for (int j = 0; j < NT; j++)
			{
				const int co = j * 8 + 2 * t;
				float v0 = acc[r][j][half * 2], v1 = acc[r][j][half * 2 + 1];
				if (EPI == EPI_RELU)
				{
					v0 = fmaxf(v0 + A.bias[co], 0.0f);
					v1 = fmaxf(v1 + A.bias[co + 1], 0.0f);
					*reinterpret_cast<uint32_t *>(A.out + pix * COUT + co) = pack_bf16x2(v0, v1);
				}
				else if (EPI == EPI_MASK)
				{
					__nv_bfloat162 m = *reinterpret_cast<const __nv_bfloat162 *>(A.mask + pix * COUT + co);
					v0 = __bfloat162float(m.x) > 0.0f ? v0 : 0.0f;
					v1 = __bfloat162float(m.y) > 0.0f ? v1 : 0.0f;
					*reinterpret_cast<uint32_t *>(A.out + pix * COUT + co) = pack_bf16x2(v0, v1);
				}
				else if (co < 4)
				{
					// Residual over the input image in [0, 1].
					float i0 = float(A.image[pix * 4 + co]) / 255.0f, i1 = float(A.image[pix * 4 + co + 1]) / 255.0f;
					v0 = v0 + A.bias[co] + i0;
					v1 = v1 + A.bias[co + 1] + i1;
					if (A.out_f32)
					{
						A.out_f32[pix * 4 + co] = v0;
						A.out_f32[pix * 4 + co + 1] = v1;
					}
					if (A.out_rgba)
					{
						A.out_rgba[pix * 4 + co] = uint8_t(rintf(fminf(fmaxf(v0, 0.0f), 1.0f) * 255.0f));
						A.out_rgba[pix * 4 + co + 1] = uint8_t(rintf(fminf(fmaxf(v1, 0.0f), 1.0f) * 255.0f));
					}
				}
			}
		}
	}
}

// Weight gradient dW[tap][co][ci] += sum_p X[p + off(tap)][ci] * dY[p][co]
// (stored in the forward layout).  Each CTA walks 16x16 pixel tiles with a
// grid stride and accumulates all nine taps in shared memory before one
// global atomic per element.
struct WgradArgs
{
	const __nv_bfloat16 *x;   // N x H x W x CIN (layer input)
	const __nv_bfloat16 *dy;  // N x H x W x COUT (gradient at the layer output, before bias)
	float *dw;                // 9 x COUT x CIN
	float *db;                // COUT
	int n, h, w;
};

template <int CIN, int COUT>
constexpr size_t wgrad_smem_bytes()
{
	return (9 * COUT * CIN + 32) * 4 + (HALO * HALO * (CIN + 8) + TILE * TILE * (COUT + 8)) * 2;
}

template <int CIN, int COUT>
__global__ void __launch_bounds__(256) wgrad_kernel(WgradArgs A)
{
	constexpr int PS = CIN + 8;
	constexpr int PD = COUT + 8;
	constexpr int MT = CIN / 16;    // m16 tiles over input channels
	constexpr int NT = COUT / 8;    // n8 tiles over output channels
	// Dynamic shared memory (over the 48 KiB static limit): the nine-tap
	// accumulator, the halo of X and the tile of dY.
	extern __shared__ __align__(16) uint8_t smem_raw[];
	float *s_dw = reinterpret_cast<float *>(smem_raw);
	float *s_db = s_dw + 9 * COUT * CIN;
	__nv_bfloat16 *s_x = reinterpret_cast<__nv_bfloat16 *>(s_db + 32);
	__nv_bfloat16 *s_dy = s_x + HALO * HALO * PS;

	const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
	for (int i = tid; i < 9 * COUT * CIN; i += 256)
		s_dw[i] = 0.0f;
	if (tid < COUT)
		s_db[tid] = 0.0f;

	const int tiles_x = (A.w + TILE - 1) / TILE, tiles_y = (A.h + TILE - 1) / TILE;
	const int tiles = tiles_x * tiles_y * A.n;
	for (int tile = blockIdx.x; tile < tiles; tile += gridDim.x)
	{
		const int img = tile / (tiles_x * tiles_y), rem = tile % (tiles_x * tiles_y);
		const int x0 = (rem % tiles_x) * TILE, y0 = (rem / tiles_x) * TILE;
		__syncthreads();
		for (int i = tid; i < HALO * HALO * (CIN / 8); i += 256)
		{
			int p = i / (CIN / 8), c = (i % (CIN / 8)) * 8;
			int gx = x0 - 1 + p % HALO, gy = y0 - 1 + p / HALO;
			uint4 v = make_uint4(0, 0, 0, 0);
			if (gx >= 0 && gy >= 0 && gx < A.w && gy < A.h)
				v = *reinterpret_cast<const uint4 *>(A.x + ((size_t(img) * A.h + gy) * A.w + gx) * CIN + c);
			*reinterpret_cast<uint4 *>(s_x + p * PS + c) = v;
		}
		for (int i = tid; i < TILE * TILE * (COUT / 8); i += 256)
		{
			int p = i / (COUT / 8), c = (i % (COUT / 8)) * 8;
			int gx = x0 + p % TILE, gy = y0 + p / TILE;
			uint4 v = make_uint4(0, 0, 0, 0);
			if (gx < A.w && gy < A.h)
				v = *reinterpret_cast<const uint4 *>(A.dy + ((size_t(img) * A.h + gy) * A.w + gx) * COUT + c);
			*reinterpret_cast<uint4 *>(s_dy + p * PD + c) = v;
		}
		__syncthreads();

		// Bias gradient: column sums of dY (pixels outside the image are zero).
		if (tid < COUT)
		{
			float s = 0.0f;
			for (int p = 0; p < TILE * TILE; p++)
				s += __bfloat162float(s_dy[p * PD + tid]);
			s_db[tid] += s;
		}

		// Warp: pixel rows 2w, 2w+1 (K = 32 pixels, two k16 steps).
		#pragma unroll 1
		for (int tap = 0; tap < 9; tap++)
		{
			const int dy = tap / 3, dx = tap % 3;
			float acc[MT][NT][4];
			#pragma unroll
			for (int m = 0; m < MT; m++)
				#pragma unroll
				for (int j = 0; j < NT; j++)
					#pragma unroll
					for (int k = 0; k < 4; k++)
						acc[m][j][k] = 0.0f;
			#pragma unroll
			for (int ks = 0; ks < 2; ks++)
			{
				const int row = warp * 2 + ks;   // the 16 pixels of one tile row are one k16 step
				// A (m = input channel, k = pixel): transposed 8x8 loads from
				// pixel-major memory.  Matrix q: pixels (q >> 1) * 8 + 0..7,
				// channels (q & 1) * 8 + 0..7.
				uint32_t a[MT][4];
				#pragma unroll
				for (int m = 0; m < MT; m++)
				{
					int q = lane >> 3, px = (q >> 1) * 8 + (lane & 7);
					const __nv_bfloat16 *p = s_x + ((row + dy) * HALO + px + dx) * PS + m * 16 + (q & 1) * 8;
					ldsm_x4_t(smem_u32(p), a[m][0], a[m][1], a[m][2], a[m][3]);
				}
				// B (k = pixel, n = output channel): transposed loads from
				// pixel-major dY; lanes 0-7 pixels 0-7, lanes 8-15 pixels 8-15.
				#pragma unroll
				for (int j = 0; j < NT; j++)
				{
					int px = ((lane >> 3) & 1) * 8 + (lane & 7);
					const __nv_bfloat16 *p = s_dy + (row * TILE + px) * PD + j * 8;
					uint32_t b0, b1;
					ldsm_x2_t(smem_u32(p), b0, b1);
					#pragma unroll
					for (int m = 0; m < MT; m++)
						mma_bf16(acc[m][j], a[m], b0, b1);
				}
			}
			// acc[m][j]: rows (ci) m*16 + g (+8), columns (co) j*8 + 2t (+1).
			const int g = lane >> 2, t = lane & 3;
			#pragma unroll
			for (int m = 0; m < MT; m++)
				#pragma unroll
				for (int j = 0; j < NT; j++)
					#pragma unroll
					for (int k = 0; k < 4; k++)
					{
						int ci = m * 16 + g + (k >> 1) * 8, co = j * 8 + 2 * t + (k & 1);
						atomicAdd(&s_dw[(tap * COUT + co) * CIN + ci], acc[m][j][k]);
					}
		}
	}
	__syncthreads();
	for (int i = tid; i < 9 * COUT * CIN; i += 256)
		atomicAdd(&A.dw[i], s_dw[i]);
	if (tid < COUT)
		atomicAdd(&A.db[tid], s_db[tid]);
}

// RGBA8 image -> BF16 16-channel input (channels 4..15 zero).
__global__ void __launch_bounds__(256) image_to_bf16_kernel(const uint8_t *img, __nv_bfloat16 *out, size_t pixels)
{
	size_t p = size_t(blockIdx.x) * blockDim.x + threadIdx.x;
	if (p >= pixels)
		return;
	uint32_t c = reinterpret_cast<const uint32_t *>(img)[p];
	uint32_t w[8];
	rgba8_to_bf16x4(c, w[0], w[1]);
	for (int i = 2; i < 8; i++)
		w[i] = 0;
	uint4 *o = reinterpret_cast<uint4 *>(out + p * 16);
	o[0] = make_uint4(w[0], w[1], w[2], w[3]);
	o[1] = make_uint4(w[4], w[5], w[6], w[7]);
}

// MSE loss over the four channels against the target image, and its
// gradient 2 (out - target) / count as BF16 16-channel input of the last
// layer's backward pass.
__global__ void __launch_bounds__(256) loss_kernel(const float *out, const uint8_t *target, size_t pixels, float scale,
                                                   __nv_bfloat16 *grad, double *loss_sum)
{
	size_t p = size_t(blockIdx.x) * blockDim.x + threadIdx.x;
	double local = 0.0;
	if (p < pixels)
	{
		uint32_t w[8] = {};
		float d[4];
		for (int k = 0; k < 4; k++)
		{
			d[k] = out[p * 4 + k] - float(target[p * 4 + k]) / 255.0f;
			local += double(d[k]) * d[k];
		}
		w[0] = pack_bf16x2(scale * d[0], scale * d[1]);
		w[1] = pack_bf16x2(scale * d[2], scale * d[3]);
		uint4 *o = reinterpret_cast<uint4 *>(grad + p * 16);
		o[0] = make_uint4(w[0], w[1], w[2], w[3]);
		o[1] = make_uint4(w[4], w[5], w[6], w[7]);
	}
	for (int o = 16; o > 0; o >>= 1)
		local += __shfl_xor_sync(0xffffffffu, local, o);
	if ((threadIdx.x & 31) == 0)
		atomicAdd(loss_sum, local);
}

// Parameter block of one layer inside the flat FP32 parameter vector:
// weights [tap][co][ci] (real sizes) then bias [co].
struct LayerOffsets
{
	int w[LAYERS], b[LAYERS];
	int total;
};

__constant__ LayerOffsets c_off;

// Adam step on the flat parameter vector, then the BF16 copies: the forward
// layout [tap][co_pad][ci_pad] and, for layers 1..5, the data-gradient layout
// [8 - tap][ci][co_pad_dgrad] (weights flipped and transposed).
__global__ void __launch_bounds__(256) adam_kernel(float *params, float *m, float *v, const float *grad, int count,
                                                   float lr, float b1, float b2, float eps, float c1, float c2)
{
	int i = blockIdx.x * blockDim.x + threadIdx.x;
	if (i >= count)
		return;
	float g = grad[i];
	float mi = b1 * m[i] + (1.0f - b1) * g;
	float vi = b2 * v[i] + (1.0f - b2) * g * g;
	m[i] = mi;
	v[i] = vi;
	params[i] -= lr * (mi / c1) / (sqrtf(vi / c2) + eps);
}

struct BfLayout
{
	__nv_bfloat16 *fwd[LAYERS];
	__nv_bfloat16 *dgrad[LAYERS];
};

__global__ void __launch_bounds__(256) pack_weights_kernel(const float *params, BfLayout L)
{
	// One thread per forward-layout element of every layer.
	int i = blockIdx.x * blockDim.x + threadIdx.x;
	for (int l = 0; l < LAYERS; l++)
	{
		int n = 9 * d_pad_out[l] * d_pad_in[l];
		if (i < n)
		{
			int tap = i / (d_pad_out[l] * d_pad_in[l]), co = (i / d_pad_in[l]) % d_pad_out[l], ci = i % d_pad_in[l];
			float w = (co < d_real_out[l] && ci < d_real_in[l])
			              ? params[c_off.w[l] + (tap * d_real_out[l] + co) * d_real_in[l] + ci] : 0.0f;
			L.fwd[l][i] = __float2bfloat16_rn(w);
		}
		if (l > 0)
		{
			// Data gradient of layer l: input channels = layer outputs padded to
			// 16 (layer 5) or 32, output channels = layer inputs (32).
			int din = l == LAYERS - 1 ? 16 : d_pad_out[l], dout = d_pad_in[l];
			int nd = 9 * dout * din;
			if (i < nd)
			{
				int tap = i / (dout * din), ci = (i / din) % dout, co = i % din;
				int src_tap = 8 - tap;
				float w = (co < d_real_out[l] && ci < d_real_in[l])
				              ? params[c_off.w[l] + (src_tap * d_real_out[l] + co) * d_real_in[l] + ci] : 0.0f;
				L.dgrad[l][i] = __float2bfloat16_rn(w);
			}
		}
	}
}

// Gradient of the last layer from a [9][8][32] (padded) wgrad buffer is
// produced directly in real layout by copying: wgrad kernels write padded
// blocks that gather_grad_kernel folds into the flat gradient vector.
__global__ void __launch_bounds__(256) gather_grad_kernel(const float *padded_w, const float *padded_b, int layer,
                                                          int cout_pad, int cin_pad, float *grad)
{
	int i = blockIdx.x * blockDim.x + threadIdx.x;
	int real_out = d_real_out[layer], real_in = d_real_in[layer];
	int nw = 9 * real_out * real_in;
	if (i < nw)
	{
		int tap = i / (real_out * real_in), co = (i / real_in) % real_out, ci = i % real_in;
		grad[c_off.w[layer] + i] = padded_w[(tap * cout_pad + co) * cin_pad + ci];
	}
	else if (i < nw + real_out)
		grad[c_off.b[layer] + (i - nw)] = padded_b[i - nw];
}


// ---------------------------------------------------------------------------
// Self-test of the tcgen05 building blocks: one CTA computes a 128x32 FP32
// tile D = A (128x32 BF16) x B (32x32 BF16)^T with two K=16 MMAs from shared
// memory in the given operand layout (0: no swizzle, 1: 64-byte swizzle) and
// writes D from tensor memory.  Inputs are small multiples of 1/8 so every
// product and sum is exact.
__device__ __forceinline__ float probe_a(uint32_t r, uint32_t k) { return float(int((r * 7u + k * 3u) % 17u) - 8) / 8.0f; }
__device__ __forceinline__ float probe_b(uint32_t n, uint32_t k) { return float(int((n * 5u + k * 11u) % 13u) - 6) / 4.0f; }

__global__ void __launch_bounds__(128) umma_probe_kernel(uint32_t mode, float *out, uint32_t *err)
{
	using namespace pgs_umma;
	extern __shared__ __align__(1024) uint8_t smem[];
	uint8_t *sa = smem;               // 128 rows x 64 B = 8 KiB
	uint8_t *sb = smem + 8192;        // 32 rows x 64 B = 2 KiB
	__shared__ uint64_t bar;
	__shared__ uint32_t tmem_slot;
	const uint32_t tid = threadIdx.x, warp = tid >> 5, lane = tid & 31u;
	const uint32_t LBO = 128, SBO = 512;
	for (uint32_t i = tid; i < 128 * 32; i += 128)
	{
		uint32_t r = i / 32, k = i % 32;
		uint32_t off = mode == 1 ? swz64_offset(r, k) : canon_offset(r, k, LBO, SBO);
		*reinterpret_cast<__nv_bfloat16 *>(sa + off) = __float2bfloat16_rn(probe_a(r, k));
		// (mode 2 never reads these operands.)
	}
	for (uint32_t i = tid; i < 32 * 32; i += 128)
	{
		uint32_t n = i / 32, k = i % 32;
		uint32_t off = mode == 1 ? swz64_offset(n, k) : canon_offset(n, k, LBO, SBO);
		*reinterpret_cast<__nv_bfloat16 *>(sb + off) = __float2bfloat16_rn(probe_b(n, k));
	}
	if (warp == 0)
		tmem_alloc(&tmem_slot, 32);
	if (tid == 0)
	{
		mbar_init(&bar, 1);
		fence_barrier_init();
	}
	fence_proxy_async();
	tc_fence_before();
	__syncthreads();
	tc_fence_after();
	const uint32_t tmem = tmem_slot;
	// Mode 2: nothing is issued, so nothing arrives on the barrier; the
	// bounded wait gives up, the error flag is set and TMEM is released.
	if (tid == 0 && mode != 2)
	{
		const uint32_t idesc = idesc_bf16_f32(128, 32);
		for (uint32_t ks = 0; ks < 2; ks++)
		{
			uint64_t ad, bd;
			if (mode == 1)
			{
				ad = smem_desc(smem_addr(sa) + ks * 32u, 16, SBO, LAYOUT_SWIZZLE_64B);
				bd = smem_desc(smem_addr(sb) + ks * 32u, 16, SBO, LAYOUT_SWIZZLE_64B);
			}
			else
			{
				ad = smem_desc(smem_addr(sa) + ks * 2u * LBO, LBO, SBO, LAYOUT_NONE);
				bd = smem_desc(smem_addr(sb) + ks * 2u * LBO, LBO, SBO, LAYOUT_NONE);
			}
			pgs_umma::mma_bf16(tmem, ad, bd, idesc, ks > 0);
		}
		mma_commit(&bar);
	}
	__syncwarp();
	bool ok = mode == 2 ? mbar_wait_limit(&bar, 0, 4096) : mbar_wait(&bar, 0);
	tc_fence_after();
	if (!ok)
	{
		if (lane == 0)
			atomicOr(err, 1u);
	}
	else
	{
		uint32_t v[32];
		tmem_ld32(tmem + ((warp * 32u) << 16), v);
		for (int c = 0; c < 32; c++)
			out[(warp * 32 + lane) * 32 + c] = __uint_as_float(v[c]);
	}
	tc_fence_before();
	__syncthreads();
	tc_fence_after();
	if (warp == 0)
		tmem_dealloc(tmem, 32);
}

// ---------------------------------------------------------------------------
// 32 -> 32 convolution on the 5th-generation tensor cores (inference and the
// forward half of training).  Persistent CTAs (one per SM) own tiles of
// 8 rows x 16 columns = 128 output pixels.  Warp-specialised pipeline:
//  - warp 0, one lane: TMA loads of three copies of each tile's 10 x 16 x 32
//    input window, shifted by dx = 0, 1, 2 columns (zero fill outside the
//    image, 64-byte swizzle), so that for every tap the 128 A rows are
//    contiguous; three input stages;
//  - the same lane issues 9 taps x 2 K-steps of tcgen05.mma (M 128, N 32,
//    K 16) into one of two 32-column FP32 accumulators in tensor memory and
//    commits to the stage's "empty" and the accumulator's "full" barriers;
//  - warps 1-4 (one per TMEM lane quarter) read the accumulator, release it,
//    add the bias, apply ReLU and store BF16 NHWC rows, overlapping the MMAs
//    of the next tile.
// The layer's weights sit in shared memory (9 x 32 x 32 BF16, 64-byte
// swizzled) for the whole launch.  Every wait is bounded and gives up when
// another warp has given up.
namespace tc
{
constexpr int ROWS = 8, COLS = 16, PIX = ROWS * COLS;
constexpr int WIN_ROWS = ROWS + 2;
constexpr int STAGES = 3, ACCS = 2;
constexpr uint32_t COPY_BYTES = WIN_ROWS * COLS * 64;      // 10240
constexpr uint32_t STAGE_BYTES = 3 * COPY_BYTES;            // 30720
constexpr uint32_t W_BYTES = 9 * 32 * 64;                   // 18432
constexpr uint32_t SMEM_BYTES = 1024 + STAGES * STAGE_BYTES + W_BYTES + 1024;
constexpr int THREADS = 160;
}

// Epilogue outputs of conv32_tc_kernel: EPI_RELU writes out = relu(acc +
// bias); EPI_MASK (the data gradient of a 32 -> 32 layer through the ReLU
// before it) writes out = acc where mask > 0, else 0.
struct TcOut
{
	__nv_bfloat16 *out;
	const __nv_bfloat16 *mask;
};

template <int EPI>
__global__ void __launch_bounds__(tc::THREADS, 2) conv32_tc_kernel(const __grid_constant__ CUtensorMap tmap,
                                                                    const __nv_bfloat16 *wt, const float *bias,
                                                                    TcOut o, int n, int h, int w, uint32_t *err)
{
	using namespace pgs_umma;
	extern __shared__ uint8_t smem_dyn[];
	uint8_t *base = reinterpret_cast<uint8_t *>((reinterpret_cast<uintptr_t>(smem_dyn) + 1023) & ~uintptr_t(1023));
	uint8_t *sw = base + tc::STAGES * tc::STAGE_BYTES;
	__shared__ uint64_t full_bar[tc::STAGES], empty_bar[tc::STAGES], acc_full[tc::ACCS], acc_empty[tc::ACCS];
	__shared__ uint32_t tmem_slot;
	__shared__ float s_bias[32];
	__shared__ volatile uint32_t s_abort;

	const uint32_t tid = threadIdx.x, warp = tid >> 5, lane = tid & 31u;
	const int tiles_x = (w + tc::COLS - 1) / tc::COLS, tiles_y = (h + tc::ROWS - 1) / tc::ROWS;
	const int tiles = tiles_x * tiles_y * n;
	griddep_launch_dependents();

	// Weights: 16-byte chunks of 8 input channels into their swizzled slots.
	for (uint32_t i = tid; i < 9 * 32 * 4; i += tc::THREADS)
	{
		uint32_t tap = i / 128, co = (i / 4) % 32, ci = (i % 4) * 8;
		*reinterpret_cast<uint4 *>(sw + tap * 2048u + swz64_offset(co, ci)) =
		    *reinterpret_cast<const uint4 *>(wt + (tap * 32u + co) * 32u + ci);
	}
	if (tid < 32)
		s_bias[tid] = EPI == EPI_MASK ? 0.0f : bias[tid];
	if (warp == 0)
		tmem_alloc(&tmem_slot, 64);
	if (tid == 0)
	{
		for (int s = 0; s < tc::STAGES; s++)
		{
			mbar_init(&full_bar[s], 1);
			mbar_init(&empty_bar[s], 1);
		}
		for (int a = 0; a < tc::ACCS; a++)
		{
			mbar_init(&acc_full[a], 1);
			mbar_init(&acc_empty[a], 4);
		}
		fence_barrier_init();
		s_abort = 0;
	}
	fence_proxy_async();
	tc_fence_before();
	__syncthreads();
	tc_fence_after();
	const uint32_t tmem = tmem_slot;
	// Weights, barriers and tensor memory are set up; the input is the
	// previous layer's output.
	griddep_wait();

	auto tile_coords = [&](int tile, int &img, int &x0, int &y0) {
		img = tile / (tiles_x * tiles_y);
		int rem = tile % (tiles_x * tiles_y);
		x0 = (rem % tiles_x) * tc::COLS;
		y0 = (rem / tiles_x) * tc::ROWS;
	};
	const int first = blockIdx.x, step = gridDim.x;
	const int mine = first < tiles ? (tiles - 1 - first) / step + 1 : 0;

	if (warp == 0)
	{
		if (lane == 0)
		{
			const uint32_t idesc = idesc_bf16_f32(128, 32);
			int loaded = 0;
			for (int i = 0; i < mine && !s_abort; i++)
			{
				// Keep up to STAGES tiles of input in flight.
				for (; loaded < mine && loaded < i + tc::STAGES; loaded++)
				{
					const int s = loaded % tc::STAGES;
					if (loaded >= tc::STAGES && !mbar_wait_or_abort(&empty_bar[s], ((loaded / tc::STAGES) - 1) & 1, &s_abort))
					{
						atomicOr(err, 1u);
						s_abort = 1;
						break;
					}
					int img, x0, y0;
					tile_coords(first + loaded * step, img, x0, y0);
					uint8_t *dst = base + s * tc::STAGE_BYTES;
					mbar_expect_tx(&full_bar[s], tc::STAGE_BYTES);
					for (int dx = 0; dx < 3; dx++)
						tma_load_4d(dst + dx * tc::COPY_BYTES, &tmap, &full_bar[s], 0, x0 - 1 + dx, y0 - 1, img);
				}
				if (s_abort)
					break;
				const int s = i % tc::STAGES, a = i % tc::ACCS;
				if (!mbar_wait_or_abort(&full_bar[s], (i / tc::STAGES) & 1, &s_abort) ||
				    (i >= tc::ACCS && !mbar_wait_or_abort(&acc_empty[a], ((i / tc::ACCS) - 1) & 1, &s_abort)))
				{
					atomicOr(err, 2u);
					s_abort = 1;
					break;
				}
				tc_fence_after();
				const uint32_t a0 = smem_addr(base + s * tc::STAGE_BYTES), b0 = smem_addr(sw);
				const uint32_t d = tmem + uint32_t(a) * 32u;
				bool acc = false;
				for (int tap = 0; tap < 9; tap++)
				{
					const int dy = tap / 3, dx = tap % 3;
					for (int ks = 0; ks < 2; ks++)
					{
						uint64_t ad = smem_desc(a0 + dx * tc::COPY_BYTES + dy * tc::COLS * 64u + ks * 32u, 16, 512,
						                        LAYOUT_SWIZZLE_64B);
						uint64_t bd = smem_desc(b0 + tap * 2048u + ks * 32u, 16, 512, LAYOUT_SWIZZLE_64B);
						pgs_umma::mma_bf16(d, ad, bd, idesc, acc);
						acc = true;
					}
				}
				mma_commit(&empty_bar[s]);
				mma_commit(&acc_full[a]);
			}
		}
		__syncwarp();
	}
	else
	{
		// Epilogue warps: warp w reads TMEM lanes 32 * (w % 4) .. + 31.
		const uint32_t quarter = warp & 3u;
		for (int i = 0; i < mine; i++)
		{
			const int a = i % tc::ACCS;
			bool ok = mbar_wait_or_abort(&acc_full[a], (i / tc::ACCS) & 1, &s_abort);
			if (!__all_sync(0xffffffffu, ok))
			{
				if (lane == 0)
					atomicOr(err, 4u);
				s_abort = 1;
				break;
			}
			tc_fence_after();
			uint32_t v[32];
			tmem_ld32(tmem + uint32_t(a) * 32u + ((quarter * 32u) << 16), v);
			tc_fence_before();
			__syncwarp();
			if (lane == 0)
				mbar_arrive(&acc_empty[a]);
			int img, x0, y0;
			tile_coords(first + i * step, img, x0, y0);
			const int pix = int(quarter * 32u + lane);
			const int gy = y0 + pix / tc::COLS, gx = x0 + pix % tc::COLS;
			const size_t pixel = (size_t(img) * h + gy) * w + gx;
			if (gx < w && gy < h)
			{
				uint32_t m[16];
				if (EPI == EPI_MASK)
				{
					const uint4 *src = reinterpret_cast<const uint4 *>(o.mask + pixel * 32);
					#pragma unroll
					for (int q = 0; q < 4; q++)
					{
						const uint4 t = src[q];
						m[4 * q] = t.x;
						m[4 * q + 1] = t.y;
						m[4 * q + 2] = t.z;
						m[4 * q + 3] = t.w;
					}
				}
				uint32_t packed[16];
				#pragma unroll
				for (int c = 0; c < 16; c++)
				{
					float lo, hi;
					if (EPI == EPI_MASK)
					{
						// Data gradient through the ReLU: keep where the layer's output was positive.
						__nv_bfloat162 mk = *reinterpret_cast<const __nv_bfloat162 *>(&m[c]);
						lo = __bfloat162float(mk.x) > 0.0f ? __uint_as_float(v[2 * c]) : 0.0f;
						hi = __bfloat162float(mk.y) > 0.0f ? __uint_as_float(v[2 * c + 1]) : 0.0f;
					}
					else
					{
						lo = fmaxf(__uint_as_float(v[2 * c]) + s_bias[2 * c], 0.0f);
						hi = fmaxf(__uint_as_float(v[2 * c + 1]) + s_bias[2 * c + 1], 0.0f);
					}
					packed[c] = pack_bf16x2(lo, hi);
				}
				uint4 *dst = reinterpret_cast<uint4 *>(o.out + pixel * 32);
				#pragma unroll
				for (int q = 0; q < 4; q++)
					dst[q] = make_uint4(packed[4 * q], packed[4 * q + 1], packed[4 * q + 2], packed[4 * q + 3]);
			}
		}
	}
	tc_fence_before();
	__syncthreads();
	tc_fence_after();
	if (warp == 0)
		tmem_dealloc(tmem, 64);
}

// Tensor map of an N x H x W x 32 BF16 activation tensor for conv32_tc_kernel:
// boxes of 32 channels x 16 columns x 10 rows, 64-byte swizzle, zero fill.
static int make_act_tmap(CUtensorMap *m, const void *ptr, int n, int h, int w)
{
	using Encode = CUresult (*)(CUtensorMap *, CUtensorMapDataType, cuuint32_t, void *, const cuuint64_t *,
	                            const cuuint64_t *, const cuuint32_t *, const cuuint32_t *, CUtensorMapInterleave,
	                            CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);
	static Encode encode = nullptr;
	if (!encode)
	{
		void *fn = nullptr;
		cudaDriverEntryPointQueryResult q;
		if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault, &q) != cudaSuccess ||
		    q != cudaDriverEntryPointSuccess || !fn)
			return PGS_ERROR_UNSUPPORTED;
		encode = reinterpret_cast<Encode>(fn);
	}
	cuuint64_t dims[4] = { 32, cuuint64_t(w), cuuint64_t(h), cuuint64_t(n) };
	cuuint64_t strides[3] = { 64, cuuint64_t(w) * 64, cuuint64_t(h) * w * 64 };
	cuuint32_t box[4] = { 32, uint32_t(tc::COLS), uint32_t(tc::WIN_ROWS), 1 };
	cuuint32_t estr[4] = { 1, 1, 1, 1 };
	CUresult r = encode(m, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 4, const_cast<void *>(ptr), dims, strides, box, estr,
	                    CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_64B, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
	                    CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
	return r == CUDA_SUCCESS ? PGS_OK : PGS_ERROR_INVALID_ARGUMENT;
}

// ---------------------------------------------------------------------------
struct Upscaler
{
	int device = 0;
	cudaStream_t stream = nullptr;      // where the upscaler's work is queued
	cudaStream_t own_stream = nullptr;  // created with the upscaler
	LayerOffsets off = {};
	float *d_params = nullptr, *d_m = nullptr, *d_v = nullptr, *d_grad = nullptr;
	float *d_wgrad = nullptr, *d_bgrad = nullptr;   // padded scratch, per layer
	size_t wgrad_stride = 9 * 32 * 32, bgrad_stride = 32;
	BfLayout bf = {};
	int adam_t = 0;
	// Activations for the current batch size.
	size_t cap_pixels = 0;
	__nv_bfloat16 *d_x0 = nullptr;              // input, 16 channels
	__nv_bfloat16 *d_act[LAYERS - 1] = {};      // outputs of layers 0..4, 32 channels
	__nv_bfloat16 *d_ga = nullptr, *d_gb = nullptr;   // gradient ping-pong, 32 channels
	__nv_bfloat16 *d_gout = nullptr;            // last-layer output gradient, 16 channels
	float *d_out = nullptr;                     // N x H x W x 4
	double *d_loss = nullptr;
	uint32_t *d_err = nullptr;
	int sm_count = 0;
	// 32 -> 32 layers: 0 = mma.sync, otherwise tcgen05 with this many
	// persistent CTAs per SM.
	int use_tc = 2;
	// Tensor maps of the activation buffers (encoded once per buffer and shape).
	struct TmapEntry
	{
		const void *ptr;
		int n, h, w;
		CUtensorMap map;
	};
	TmapEntry tmaps[12] = {};
	int tmap_count = 0;

	int act_tmap(const void *ptr, int n, int h, int w, CUtensorMap *&out)
	{
		for (int i = 0; i < tmap_count; i++)
			if (tmaps[i].ptr == ptr && tmaps[i].n == n && tmaps[i].h == h && tmaps[i].w == w)
			{
				out = &tmaps[i].map;
				return PGS_OK;
			}
		TmapEntry &e = tmaps[tmap_count < 12 ? tmap_count++ : 11];
		int r = make_act_tmap(&e.map, ptr, n, h, w);
		if (r)
			return r;
		e.ptr = ptr;
		e.n = n;
		e.h = h;
		e.w = w;
		out = &e.map;
		return PGS_OK;
	}

	int init(int dev)
	{
		device = dev;
		UP_TRY(cudaSetDevice(device));
		UP_TRY(cudaStreamCreateWithFlags(&own_stream, cudaStreamNonBlocking));
		stream = own_stream;
		UP_TRY(cudaDeviceGetAttribute(&sm_count, cudaDevAttrMultiProcessorCount, device));
		int o = 0;
		for (int l = 0; l < LAYERS; l++)
		{
			off.w[l] = o;
			o += 9 * REAL_OUT[l] * REAL_IN[l];
			off.b[l] = o;
			o += REAL_OUT[l];
		}
		off.total = o;
		UP_TRY(cudaMemcpyToSymbol(c_off, &off, sizeof(off)));
		size_t n = size_t(off.total);
		UP_TRY(cudaMalloc(&d_params, n * 4));
		UP_TRY(cudaMalloc(&d_m, n * 4));
		UP_TRY(cudaMalloc(&d_v, n * 4));
		UP_TRY(cudaMalloc(&d_grad, n * 4));
		UP_TRY(cudaMemset(d_params, 0, n * 4));
		UP_TRY(cudaMemset(d_m, 0, n * 4));
		UP_TRY(cudaMemset(d_v, 0, n * 4));
		UP_TRY(cudaMalloc(&d_wgrad, LAYERS * wgrad_stride * 4));
		UP_TRY(cudaMalloc(&d_bgrad, LAYERS * bgrad_stride * 4));
		for (int l = 0; l < LAYERS; l++)
		{
			UP_TRY(cudaMalloc(&bf.fwd[l], size_t(9) * PAD_OUT[l] * PAD_IN[l] * 2));
			UP_TRY(cudaMalloc(&bf.dgrad[l], size_t(9) * 32 * 32 * 2));
		}
		UP_TRY(cudaMalloc(&d_loss, sizeof(double)));
		UP_TRY(cudaMalloc(&d_err, sizeof(uint32_t)));
		UP_TRY(cudaMemset(d_err, 0, sizeof(uint32_t)));
		UP_TRY(cudaFuncSetAttribute(conv32_tc_kernel<EPI_RELU>, cudaFuncAttributeMaxDynamicSharedMemorySize,
		                            int(tc::SMEM_BYTES)));
		UP_TRY(cudaFuncSetAttribute(conv32_tc_kernel<EPI_MASK>, cudaFuncAttributeMaxDynamicSharedMemorySize,
		                            int(tc::SMEM_BYTES)));
		return PGS_OK;
	}

	void destroy()
	{
		cudaSetDevice(device);
		if (stream)
			cudaStreamSynchronize(stream);
		cudaFree(d_params);
		cudaFree(d_m);
		cudaFree(d_v);
		cudaFree(d_grad);
		cudaFree(d_wgrad);
		cudaFree(d_bgrad);
		for (int l = 0; l < LAYERS; l++)
		{
			cudaFree(bf.fwd[l]);
			cudaFree(bf.dgrad[l]);
		}
		free_acts();
		cudaFree(d_loss);
		cudaFree(d_err);
		if (own_stream)
			cudaStreamDestroy(own_stream);
	}

	// Later work goes to `s` (the upscaler's own stream when null), after
	// what is queued on the current one.
	int set_stream(cudaStream_t s)
	{
		UP_TRY(cudaSetDevice(device));
		UP_TRY(cudaStreamSynchronize(stream));
		stream = s ? s : own_stream;
		return PGS_OK;
	}

	void free_acts()
	{
		cudaFree(d_x0);
		for (auto &a : d_act)
			cudaFree(a);
		cudaFree(d_ga);
		cudaFree(d_gb);
		cudaFree(d_gout);
		cudaFree(d_out);
		d_x0 = d_ga = d_gb = d_gout = nullptr;
		for (auto &a : d_act)
			a = nullptr;
		d_out = nullptr;
		cap_pixels = 0;
	}

	int ensure(size_t pixels)
	{
		if (pixels <= cap_pixels)
			return PGS_OK;
		UP_TRY(cudaStreamSynchronize(stream));
		free_acts();
		tmap_count = 0;
		UP_TRY(cudaMalloc(&d_x0, pixels * 16 * 2));
		for (auto &a : d_act)
			UP_TRY(cudaMalloc(&a, pixels * 32 * 2));
		UP_TRY(cudaMalloc(&d_ga, pixels * 32 * 2));
		UP_TRY(cudaMalloc(&d_gb, pixels * 32 * 2));
		UP_TRY(cudaMalloc(&d_gout, pixels * 16 * 2));
		UP_TRY(cudaMalloc(&d_out, pixels * 4 * 4));
		cap_pixels = pixels;
		return PGS_OK;
	}

	int pack()
	{
		int n = 9 * 32 * 32;
		pack_weights_kernel<<<(n + 255) / 256, 256, 0, stream>>>(d_params, bf);
		UP_TRY(cudaGetLastError());
		return PGS_OK;
	}

	int set_params(const float *host, size_t count)
	{
		if (count != size_t(off.total))
			return PGS_ERROR_INVALID_ARGUMENT;
		UP_TRY(cudaMemcpyAsync(d_params, host, count * 4, cudaMemcpyHostToDevice, stream));
		UP_TRY(cudaMemsetAsync(d_m, 0, count * 4, stream));
		UP_TRY(cudaMemsetAsync(d_v, 0, count * 4, stream));
		adam_t = 0;
		int r = pack();
		if (r)
			return r;
		UP_TRY(cudaStreamSynchronize(stream));
		return PGS_OK;
	}

	int get(const float *src, float *host, size_t count)
	{
		if (count != size_t(off.total))
			return PGS_ERROR_INVALID_ARGUMENT;
		UP_TRY(cudaMemcpyAsync(host, src, count * 4, cudaMemcpyDeviceToHost, stream));
		UP_TRY(cudaStreamSynchronize(stream));
		return PGS_OK;
	}

	// 3x3 convolution of a 32-channel tensor into 32 accumulator channels on
	// tcgen05 (conv32_tc_kernel) with the given epilogue.
	template <int EPI>
	int conv_tc(const ConvArgs &a, bool pdl = false)
	{
		CUtensorMap *m = nullptr;
		int r = act_tmap(a.in, a.n, a.h, a.w, m);
		if (r)
			return r;
		int tiles = ((a.w + tc::COLS - 1) / tc::COLS) * ((a.h + tc::ROWS - 1) / tc::ROWS) * a.n;
		int grid = std::min(tiles, sm_count * use_tc);
		TcOut o = { a.out, a.mask };
		return launch(conv32_tc_kernel<EPI>, dim3(grid), dim3(tc::THREADS), tc::SMEM_BYTES, pdl, *m, a.wt, a.bias, o,
		              a.n, a.h, a.w, d_err);
	}

	template <int CIN, int COUT, int EPI>
	int conv(const ConvArgs &a, bool pdl = false)
	{
		dim3 grid((a.w + TILE - 1) / TILE, (a.h + TILE - 1) / TILE, a.n);
		return launch(conv3x3_kernel<CIN, COUT, EPI>, grid, dim3(256), 0, pdl, a);
	}

	// Launch on the upscaler's stream; pdl: the kernel may start while the
	// one before it in the stream runs (it waits for it in griddep_wait).
	template <typename... KArgs, typename... Args>
	int launch(void (*kernel)(KArgs...), dim3 grid, dim3 block, size_t smem, bool pdl, Args &&...args)
	{
		cudaLaunchConfig_t cfg = {};
		cfg.gridDim = grid;
		cfg.blockDim = block;
		cfg.dynamicSmemBytes = smem;
		cfg.stream = stream;
		cudaLaunchAttribute attr[1];
		attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
		attr[0].val.programmaticStreamSerializationAllowed = 1;
		cfg.attrs = attr;
		cfg.numAttrs = pdl ? 1 : 0;
		UP_TRY(cudaLaunchKernelEx(&cfg, kernel, std::forward<Args>(args)...));
		return PGS_OK;
	}

	// Forward pass of `n` images of h x w RGBA8 (device memory).  The FP32
	// result stays in d_out; out_rgba (device, optional) gets it clamped and
	// rounded to RGBA8.
	// keep_input: the 16-channel BF16 input is kept in d_x0 (training needs
	// it for the first layer's weight gradient); otherwise the first layer
	// reads the RGBA8 image directly.
	int forward(const uint8_t *d_img, int n, int h, int w, uint8_t *out_rgba, bool keep_input)
	{
		size_t pixels = size_t(n) * h * w;
		int r = ensure(pixels);
		if (r)
			return r;
		if (keep_input)
		{
			image_to_bf16_kernel<<<unsigned((pixels + 255) / 256), 256, 0, stream>>>(d_img, d_x0, pixels);
			UP_TRY(cudaGetLastError());
		}
		ConvArgs k = {};
		k.n = n;
		k.h = h;
		k.w = w;
		for (int l = 0; l < LAYERS; l++)
		{
			k.in = l == 0 ? d_x0 : d_act[l - 1];
			k.in_rgba = l == 0 && !keep_input ? d_img : nullptr;
			k.wt = bf.fwd[l];
			k.bias = d_params + off.b[l];
			if (l < LAYERS - 1)
			{
				k.out = d_act[l];
				// The 4 -> 32 layer stays on mma.sync: on tcgen05 it would be a
				// 32 -> 32 layer with 28 zero input channels, which measured slower.
				// Inference launches every layer after the first with
				// programmatic dependent launch: its set-up overlaps the
				// previous layer's last wave.
				const bool pdl = !keep_input && l > 0;
				if (l == 0)
					r = conv<16, 32, EPI_RELU>(k);
				else if (use_tc)
					r = conv_tc<EPI_RELU>(k, pdl);
				else
					r = conv<32, 32, EPI_RELU>(k, pdl);
			}
			else
			{
				// 32 -> 4 likewise (N = 32 with 28 zero output channels).
				k.out = nullptr;
				k.image = d_img;
				k.out_f32 = d_out;
				k.out_rgba = out_rgba;
				r = conv<32, 8, EPI_LAST>(k, !keep_input);
			}
			if (r)
				return r;
		}
		return PGS_OK;
	}

	template <int CIN, int COUT>
	int wgrad(const __nv_bfloat16 *x, const __nv_bfloat16 *dy, int layer, int n, int h, int w)
	{
		WgradArgs a = { x, dy, d_wgrad + layer * wgrad_stride, d_bgrad + layer * bgrad_stride, n, h, w };
		int tiles = ((w + TILE - 1) / TILE) * ((h + TILE - 1) / TILE) * n;
		int grid = std::min(tiles, sm_count * 2);
		constexpr size_t smem = wgrad_smem_bytes<CIN, COUT>();
		UP_TRY(cudaFuncSetAttribute(wgrad_kernel<CIN, COUT>, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem)));
		wgrad_kernel<CIN, COUT><<<grid, 256, smem, stream>>>(a);
		UP_TRY(cudaGetLastError());
		return PGS_OK;
	}

	// Loss and parameter gradient (into d_grad) for a batch; *loss = mean
	// squared error over all four channels.
	int backward(const uint8_t *d_img, const uint8_t *d_target, int n, int h, int w, double *loss)
	{
		int r = forward(d_img, n, h, w, nullptr, true);
		if (r)
			return r;
		size_t pixels = size_t(n) * h * w;
		UP_TRY(cudaMemsetAsync(d_loss, 0, sizeof(double), stream));
		UP_TRY(cudaMemsetAsync(d_wgrad, 0, LAYERS * wgrad_stride * 4, stream));
		UP_TRY(cudaMemsetAsync(d_bgrad, 0, LAYERS * bgrad_stride * 4, stream));
		float scale = 2.0f / float(pixels * 4);
		loss_kernel<<<unsigned((pixels + 255) / 256), 256, 0, stream>>>(d_out, d_target, pixels, scale, d_gout, d_loss);
		UP_TRY(cudaGetLastError());
		// Layer 5: weight gradient from the 16-channel output gradient, data
		// gradient into layer 4's output through its ReLU.
		if ((r = wgrad<32, 16>(d_act[4], d_gout, 5, n, h, w)))
			return r;
		ConvArgs k = {};
		k.n = n;
		k.h = h;
		k.w = w;
		k.in = d_gout;
		k.wt = bf.dgrad[5];
		k.mask = d_act[4];
		k.out = d_ga;
		if ((r = conv<16, 32, EPI_MASK>(k)))
			return r;
		__nv_bfloat16 *g = d_ga, *g2 = d_gb;
		for (int l = 4; l >= 1; l--)
		{
			if ((r = wgrad<32, 32>(d_act[l - 1], g, l, n, h, w)))
				return r;
			k.in = g;
			k.wt = bf.dgrad[l];
			k.mask = d_act[l - 1];
			k.out = g2;
			if ((r = use_tc ? conv_tc<EPI_MASK>(k) : conv<32, 32, EPI_MASK>(k)))
				return r;
			std::swap(g, g2);
		}
		if ((r = wgrad<16, 32>(d_x0, g, 0, n, h, w)))
			return r;
		for (int l = 0; l < LAYERS; l++)
		{
			int cout_pad = l == LAYERS - 1 ? 16 : 32, cin_pad = PAD_IN[l];
			int count = 9 * REAL_OUT[l] * REAL_IN[l] + REAL_OUT[l];
			gather_grad_kernel<<<(count + 255) / 256, 256, 0, stream>>>(d_wgrad + l * wgrad_stride,
			                                                            d_bgrad + l * bgrad_stride, l, cout_pad,
			                                                            cin_pad, d_grad);
			UP_TRY(cudaGetLastError());
		}
		if (loss)
		{
			double s = 0.0;
			UP_TRY(cudaMemcpyAsync(&s, d_loss, sizeof(double), cudaMemcpyDeviceToHost, stream));
			UP_TRY(cudaStreamSynchronize(stream));
			*loss = s / double(pixels * 4);
		}
		return PGS_OK;
	}

	int step(float lr)
	{
		adam_t++;
		const float b1 = 0.9f, b2 = 0.999f;
		float c1 = 1.0f - std::pow(b1, float(adam_t)), c2 = 1.0f - std::pow(b2, float(adam_t));
		adam_kernel<<<(off.total + 255) / 256, 256, 0, stream>>>(d_params, d_m, d_v, d_grad, off.total, lr, b1, b2, 1e-8f,
		                                                         c1, c2);
		UP_TRY(cudaGetLastError());
		return pack();
	}
};
} // namespace pgs_up

using pgs_up::Upscaler;

extern "C" {
void *pgs_upscaler_create(int device, int *status)
{
	int dummy;
	if (!status)
		status = &dummy;
	int count = 0;
	if (cudaGetDeviceCount(&count) != cudaSuccess || count == 0)
	{
		*status = PGS_ERROR_NO_DEVICE;
		return nullptr;
	}
	auto *u = new (std::nothrow) Upscaler();
	if (!u)
	{
		*status = PGS_ERROR_OUT_OF_MEMORY;
		return nullptr;
	}
	int r = u->init(device);
	if (r)
	{
		u->destroy();
		delete u;
		*status = r;
		return nullptr;
	}
	*status = PGS_OK;
	return u;
}

void pgs_upscaler_destroy(void *up)
{
	if (!up)
		return;
	static_cast<Upscaler *>(up)->destroy();
	delete static_cast<Upscaler *>(up);
}

uint32_t pgs_upscaler_param_count(void *up) { return up ? uint32_t(static_cast<Upscaler *>(up)->off.total) : 0; }

int pgs_upscaler_set_params(void *up, const float *params, uint32_t count)
{
	return up && params ? static_cast<Upscaler *>(up)->set_params(params, count) : PGS_ERROR_INVALID_ARGUMENT;
}

int pgs_upscaler_get_params(void *up, float *params, uint32_t count)
{
	if (!up || !params)
		return PGS_ERROR_INVALID_ARGUMENT;
	Upscaler *u = static_cast<Upscaler *>(up);
	return u->get(u->d_params, params, count);
}

int pgs_upscaler_get_gradient(void *up, float *grad, uint32_t count)
{
	if (!up || !grad)
		return PGS_ERROR_INVALID_ARGUMENT;
	Upscaler *u = static_cast<Upscaler *>(up);
	return u->get(u->d_grad, grad, count);
}

int pgs_upscaler_forward(void *up, const void *d_images, uint32_t n, uint32_t h, uint32_t w, void *d_out_rgba)
{
	if (!up || !d_images || !n || !h || !w)
		return PGS_ERROR_INVALID_ARGUMENT;
	Upscaler *u = static_cast<Upscaler *>(up);
	cudaSetDevice(u->device);
	return u->forward(static_cast<const uint8_t *>(d_images), int(n), int(h), int(w), static_cast<uint8_t *>(d_out_rgba),
	                  false);
}

int pgs_upscaler_backward(void *up, const void *d_images, const void *d_targets, uint32_t n, uint32_t h, uint32_t w,
                          double *loss)
{
	if (!up || !d_images || !d_targets || !n || !h || !w)
		return PGS_ERROR_INVALID_ARGUMENT;
	Upscaler *u = static_cast<Upscaler *>(up);
	cudaSetDevice(u->device);
	return u->backward(static_cast<const uint8_t *>(d_images), static_cast<const uint8_t *>(d_targets), int(n), int(h),
	                   int(w), loss);
}

int pgs_upscaler_adam_step(void *up, float lr)
{
	if (!up)
		return PGS_ERROR_INVALID_ARGUMENT;
	Upscaler *u = static_cast<Upscaler *>(up);
	cudaSetDevice(u->device);
	return u->step(lr);
}

int pgs_umma_selftest(int device, uint32_t mode, float *out_host)
{
	if (!out_host || mode > 2)
		return PGS_ERROR_INVALID_ARGUMENT;
	UP_TRY(cudaSetDevice(device));
	float *d_out = nullptr;
	uint32_t *d_err = nullptr;
	UP_TRY(cudaMalloc(&d_out, 128 * 32 * 4));
	UP_TRY(cudaMalloc(&d_err, 4));
	UP_TRY(cudaMemset(d_out, 0, 128 * 32 * 4));
	UP_TRY(cudaMemset(d_err, 0, 4));
	// Generous allocation: every address the descriptors can form stays inside.
	const int smem = 96 * 1024;
	UP_TRY(cudaFuncSetAttribute(pgs_up::umma_probe_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, smem));
	pgs_up::umma_probe_kernel<<<1, 128, smem>>>(mode, d_out, d_err);
	cudaError_t e = cudaDeviceSynchronize();
	uint32_t err = 0;
	if (e == cudaSuccess)
		e = cudaMemcpy(out_host, d_out, 128 * 32 * 4, cudaMemcpyDeviceToHost);
	if (e == cudaSuccess)
		e = cudaMemcpy(&err, d_err, 4, cudaMemcpyDeviceToHost);
	cudaFree(d_out);
	cudaFree(d_err);
	if (e != cudaSuccess)
		return PGS_ERROR_CUDA;
	return err ? PGS_ERROR_DEVICE_FLAG : PGS_OK;
}

int pgs_upscaler_set_tensor_path(void *up, int tcgen05)
{
	if (!up)
		return PGS_ERROR_INVALID_ARGUMENT;
	if (tcgen05 < 0 || tcgen05 > 2)
		return PGS_ERROR_INVALID_ARGUMENT;
	static_cast<Upscaler *>(up)->use_tc = tcgen05;
	return PGS_OK;
}

int pgs_upscaler_get_error(void *up, uint32_t *flags)
{
	if (!up || !flags)
		return PGS_ERROR_INVALID_ARGUMENT;
	Upscaler *u = static_cast<Upscaler *>(up);
	UP_TRY(cudaMemcpyAsync(flags, u->d_err, sizeof(uint32_t), cudaMemcpyDeviceToHost, u->stream));
	UP_TRY(cudaStreamSynchronize(u->stream));
	return *flags ? PGS_ERROR_DEVICE_FLAG : PGS_OK;
}

void *pgs_upscaler_stream(void *up) { return up ? static_cast<void *>(static_cast<Upscaler *>(up)->stream) : nullptr; }

int pgs_upscaler_set_stream(void *up, void *stream)
{
	if (!up)
		return PGS_ERROR_INVALID_ARGUMENT;
	return static_cast<Upscaler *>(up)->set_stream(static_cast<cudaStream_t>(stream));
}

int pgs_upscaler_synchronize(void *up)
{
	if (!up)
		return PGS_ERROR_INVALID_ARGUMENT;
	return cudaStreamSynchronize(static_cast<Upscaler *>(up)->stream) == cudaSuccess ? PGS_OK : PGS_ERROR_CUDA;
}
}
