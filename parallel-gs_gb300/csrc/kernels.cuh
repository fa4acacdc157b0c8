// kernels.cuh -- sm_103a kernels of the GS backend.
//
//   setup_kernel     one thread per primitive: edge planes, reciprocal area,
//                    attribute deltas, bounding box (triangle_setup.comp)
//   bin_kernel       32 primitives per CTA: per-coarse-tile membership and
//                    super-sampling flags (binning.comp), and the primitive's
//                    bit in the bitmask of every 8x8 sub-tile it may touch;
//                    the bitmask keeps primitive order without any sort
//   shade_kernel     one CTA per 8x8-pixel sub-tile of a coarse tile, one
//                    thread per pixel sample; walks the tile's primitives in
//                    order with the deferred-shading logic of ubershader.comp
//   upload_kernel    host->local and local->local transfers into swizzled VRAM
//   clut_kernel      CLUT instance load (clut_write.comp)
//
// All floating-point steps use explicit round-to-nearest intrinsics so that
// no multiply-add is contracted; the build also passes -fmad=false.
#pragma once

#include "gs_defs.h"
#include "pgs.h"

#include <cuda_runtime.h>
#include <stdint.h>

namespace pgs
{
// ---------------------------------------------------------------------------
// Device records.
struct __align__(16) PrimSetup
{
	int32_t a[3];
	float inv_area;
	int32_t b[3];
	float error_i;
	int32_t c[3];
	float error_j;
	int32_t bb[4];
	uint32_t z[4];
};
static_assert(sizeof(PrimSetup) == 80, "PrimSetup layout");

// Interpolation terms per primitive: value at the first vertex and the
// differences to the other two, for S T Q FOG and for the unorm colour.
struct __align__(16) TransformedAttr
{
	float stqf0[4];
	float stqf1[4];
	float stqf2[4];
	float rgba0[4];
	float rgba1[4];
	float rgba2[4];
};
static_assert(sizeof(TransformedAttr) == 96, "TransformedAttr layout");

// Decoded framebuffer instance for the shading kernels.
struct DevInstance
{
	uint32_t fb_base, fb_stride, fb_psm;
	uint32_t zb_base, zb_psm; // zb_psm == 0xffffffff when not Z sensitive
	int32_t base_x, base_y;
	uint32_t tiles_w, tiles_h;
	uint32_t rate_x_log2, rate_y_log2;
	uint32_t preserve_samples;
	uint32_t instance;
	uint32_t prim_lo, prim_count; // primitive range of this dispatch
	uint32_t mask_words;          // bitmask words per 8x8 sub-tile (1 bit per primitive)
	uint32_t summary_words;       // summary words per sub-tile (1 bit per mask word)
	uint32_t sub_w, sub_h;        // 8x8 sub-tiles per row / column
	int32_t snap_mask_y;          // raster snap of rows: half the sample pitch when field rendering
	uint32_t force_ss;            // field rendering: every covered tile super-sampled
	uint32_t blend_demote;        // primitives per coarse tile that demote a blended tile, 0 = off
};

// Linear RGBA8 image decoded from swizzled VRAM + CLUT for one mip level of
// one texture of a pass (the role of the reference's texture cache,
// upload.comp:108-229); slot l of texture t is entry t * TEX_SLOTS + l: mip
// level l, or for a super-sampled texture layer l (0: single-sampled image,
// s + 1: sample s).
constexpr uint32_t TEX_LEVELS = 7;
constexpr uint32_t TEX_SLOTS = 17;
// Phase LUT of super-sampled texture filtering: 64 x 64 (x, y) pairs for
// bilinear, then 32 x 32 sample ids for nearest.
constexpr uint32_t PHASE_LUT_WORDS = 64 * 64 * 2 + 32 * 32;

// Mean position of the samples inside a pixel per sampling grid
// (get_average_sampling_offset, utils.h:108-126).
__host__ __device__ inline float average_sampling_offset(uint32_t rx, uint32_t ry)
{
	if (rx == ry)
		return ry == 0 ? 0.0f : (ry == 1 ? 0.25f : (ry == 2 ? 0.375f : 0.4375f));
	if (rx == 0 && ry == 1)
		return 0.25f;
	if (rx == 1 && ry == 2)
		return 0.375f;
	if (rx == 0 && ry == 2)
		return 0.375f;
	if (rx == 1 && ry == 3)
		return 0.4375f;
	return 0.0f;
}

__host__ __device__ inline uint32_t texture_slots(const pgs_texture_desc &t)
{
	return t.samples > 1 ? t.samples + 1 : (t.levels > 1 ? t.levels : 1u);
}

struct TexImage
{
	uint32_t offset; // first texel in PassParams::texels
	uint32_t ext_u, ext_v;
	uint32_t padding;
};

// Flat-primitive depth buckets found by triangle setup in a super-sampled pass
// (SingleSampleHeuristic, gs/shaders/data_structures.h:190-195).  Each of the
// 256 buckets covers 2^16 (2^8 for 16-bit Z) depth values.
struct SsHeuristic
{
	uint32_t bucket_count;
	uint32_t active[8];
	uint32_t bucket[256];
};

// Per-instance depth quantisation for the heuristic
// (dispatch_single_sample_heuristic, gs/gs_renderer.cpp:1979-2039).
struct HeuristicParams
{
	uint32_t z_shift_bucket[8];
	uint32_t z_shift[8];
	uint32_t z_max[8];
	uint32_t instance_mask;
};

// Decision of the heuristic for one primitive, applied after every bucket has
// been evaluated against the states triangle setup produced.
constexpr uint8_t HEURISTIC_SET_SNAP_RASTER = 1;
constexpr uint8_t HEURISTIC_CLEAR_SNAP_ATTRIBUTE = 2;

struct PassParams
{
	// Textures [snap_limit[k - 1], snap_limit[k]) are decoded from
	// snap_vram[k], the rest from vram.
	const uint8_t *snap_vram[PGS_MAX_VRAM_SNAPSHOTS];
	uint32_t snap_limit[PGS_MAX_VRAM_SNAPSHOTS];
	uint32_t num_snaps;
	const pgs_vertex_position *pos;
	const pgs_vertex_attribute *attr;
	pgs_primitive_attribute *prims;
	const pgs_state_vector *states;
	const pgs_texture_desc *textures;
	const TexImage *tex_images;
	uint32_t *texels;
	PrimSetup *setup;
	TransformedAttr *tattr;
	uint32_t num_prims;
	uint32_t num_states, num_textures;
	uint32_t max_tex_levels;      // largest slot count (mip levels or sample layers) of the pass's textures
	uint32_t rp_is_blur_mask;     // per instance: the pass looks like a blur kernel (render_pass_instance_is_deduced_blur)
	uint32_t force_linear_ss;     // FORCE_LINEAR_SUPER_SAMPLE: field rendering with super-sampled textures
	const uint32_t *phase_lut;    // PHASE_LUT_WORDS words
	uint32_t tile_size_log2;
	uint32_t has_aa1, has_scanmsk, has_ss_reference;
	uint32_t setup_rate_x_log2, setup_rate_y_log2;
	uint32_t opaque_fbmask[8];
	uint8_t *vram;
	// Depth reads come from this snapshot of all VRAM planes when set
	// (frame and depth buffer aliased), else from vram.
	const uint8_t *zcache;
	const uint16_t *clut;
	const float *rcp_float_lut;
	const float *unorm_lut;
	uint32_t *error_flags;
	unsigned long long *fragment_counter;
	// 4 bits per instance: flat-primitive bucket shift / 8 (z_shift_to_bucket,
	// gs/gs_renderer.cpp:1914-1934).
	uint32_t packed_z_shift;
	SsHeuristic *heuristic;
	uint8_t *heuristic_action;
};

// Per-tile flag bits written by bin_kernel.
constexpr uint32_t TILE_NONEMPTY = 1u << 0;
constexpr uint32_t TILE_REQ_SS = 1u << 1;
constexpr uint32_t TILE_REQ_SS_ZW = 1u << 2;
constexpr uint32_t TILE_HAS_ZW = 1u << 3;
// Primitives binned to the tile, counted from this bit when blend demotion is on.
constexpr uint32_t TILE_COUNT_SHIFT = 8;

constexpr uint32_t ERROR_FLAG_TILE_OVERFLOW = 1u << 0;

__constant__ uint8_t c_rcp_tab[256];

// Occupancy target of the shading kernels in 256-thread units per SM: 4 means
// at most 64 registers per thread for the 1x..4x variants.  The plain 4x
// variant (no AA1, no mipmaps) asks for 5 CTAs (48 registers, a few spills):
// measured on the C2 frame, 3 CTAs 1.24 ms, 4 CTAs 1.10 ms, 5 CTAs 1.09 ms.
// The AA1 / mipmap variants, larger, stay at 4.
#ifndef PGS_SHADE_OCC
#define PGS_SHADE_OCC 4
#endif
#define PGS_SHADE_MIN_BLOCKS(NS, LARGE) \
	((NS) == 4 && !(LARGE) ? PGS_SHADE_OCC + 1 : (PGS_SHADE_OCC * 4 / (NS) > 0 ? PGS_SHADE_OCC * 4 / (NS) : 1))

// ---------------------------------------------------------------------------
// Scalar helpers.
__device__ __forceinline__ float fmul(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ float fadd(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ float fsub(float a, float b) { return __fsub_rn(a, b); }
__device__ __forceinline__ float u2f(uint32_t u) { return __uint_as_float(u); }
__device__ __forceinline__ uint32_t f2u(float f) { return __float_as_uint(f); }

__device__ __forceinline__ int32_t idot3(const int32_t p[3], int32_t x, int32_t y)
{
	return int32_t(uint32_t(p[0]) * uint32_t(x) + uint32_t(p[1]) * uint32_t(y) + uint32_t(p[2]));
}

// Reciprocal of a 32-bit fixed-point area: table seed plus two Newton steps in
// 32-bit fixed point, quantised to FP32 (rcp_fixed, math_utils.h:27-61).
__device__ __forceinline__ float rcp_fixed(uint32_t b)
{
	int lz = __clz(b);
	uint32_t nb = b << lz;
	uint32_t rcp = uint32_t(c_rcp_tab[(nb >> 23) & 0xffu]) | 0x100u;
	uint32_t f = (rcp * rcp) << 14;
	uint32_t p = __umulhi(f, nb);
	rcp = (rcp << 23) - p;
	rcp <<= 1;
	p = __umulhi(rcp, nb);
	rcp = __umulhi(rcp, 0u - p);
	rcp = (rcp + 64u) >> 7;
	rcp -= 1u << 23;
	rcp += uint32_t(127 - 32 + lz) << 23;
	return u2f(rcp);
}

// Reciprocal by table seed + 4 Newton-Raphson steps (rcp_float, math_utils.h:65-101).
__device__ __forceinline__ float rcp_float(float v, const float *lut)
{
	uint32_t u = f2u(v);
	int e = int((u >> 23) & 0xffu);
	if (e == 0)
		return u2f(0x7f800000u);
	int shifted = 127 - e;
	float x = lut[(u >> 15) & 0xffu];
	u = (u & ((1u << 23) - 1u)) | (127u << 23);
	float a = u2f(u);
	#pragma unroll
	for (int it = 0; it < 4; it++)
	{
		float x2 = fmul(x, 2.0f);
		float xs = fmul(x, x);
		float xsa = fmul(xs, a);
		x = fsub(x2, xsa);
	}
	return ldexpf(x, shifted);
}

__device__ __forceinline__ bool tie_break(int32_t ex, int32_t ey) { return ey > 0 || (ey == 0 && ex < 0); }

__device__ __forceinline__ bool order_less(int32_t ax, int32_t ay, int32_t bx, int32_t by, uint32_t az, uint32_t bz)
{
	if (bz != az) return az < bz;
	if (by != ay) return ay < by;
	return ax < bx;
}

template <typename T>
__device__ __forceinline__ void dswap(T &a, T &b) { T t = a; a = b; b = t; }

// ---------------------------------------------------------------------------
// K1: triangle setup.
__device__ __forceinline__ float unorm8_lut(const float *lut, uint32_t c, int ch) { return __ldg(lut + ((c >> (8 * ch)) & 0xffu)); }

// Colour terms of the shading interpolation c0 + (c1 - c0) i + (c2 - c0) j,
// per channel in unorm floats.
__device__ __forceinline__ void set_color_terms(const PassParams &P, TransformedAttr &ta, uint32_t r0, uint32_t r1,
                                                uint32_t r2)
{
	#pragma unroll
	for (int k = 0; k < 4; k++)
	{
		const float c0 = unorm8_lut(P.unorm_lut, r0, k), c1 = unorm8_lut(P.unorm_lut, r1, k);
		const float c2 = unorm8_lut(P.unorm_lut, r2, k);
		ta.rgba0[k] = c0;
		ta.rgba1[k] = fsub(c1, c0);
		ta.rgba2[k] = fsub(c2, c0);
	}
}

__global__ void __launch_bounds__(128) setup_kernel(PassParams P)
{
	uint32_t index = blockIdx.x * blockDim.x + threadIdx.x;
	if (index >= P.num_prims)
		return;

	pgs_primitive_attribute pa = P.prims[index];
	PrimSetup out;
	TransformedAttr ta;
	const int sry = int(P.setup_rate_y_log2);

	int order0 = 0, order1 = 1, order2 = 2;
	uint32_t st = pa.state;
	bool parallelogram = (st >> STATE_BIT_PARALLELOGRAM) & 1;
	bool perspective = (st >> STATE_BIT_PERSPECTIVE) & 1;
	bool iip = (st >> STATE_BIT_IIP) & 1;
	bool fix = (st >> STATE_BIT_FIX) & 1;
	bool sprite = (st >> STATE_BIT_SPRITE) & 1;
	bool line = (st >> STATE_BIT_LINE) & 1;
	bool multisample = (st >> STATE_BIT_MULTISAMPLE) & 1;
	uint32_t provoking = (st >> STATE_PARALLELOGRAM_PROVOKING_OFFSET) & 3u;
	uint32_t opaque_fbmask = P.opaque_fbmask[(st >> STATE_VERTEX_RENDER_PASS_INSTANCE_OFFSET) & 7u];

	pgs_vertex_position v0 = P.pos[3 * index], v1 = P.pos[3 * index + 1], v2 = P.pos[3 * index + 2];
	int32_t ax = v0.x, ay = v0.y, bx = v1.x, by = v1.y, cx = v2.x, cy = v2.y;
	uint32_t za = v0.z, zb = v1.z, zc = v2.z;

	if (line)
	{
		bool sax = (ax & 15) == 0, say = (ay & 15) == 0, sbx = (bx & 15) == 0, sby = (by & 15) == 0;
		if ((sax || sbx) && bx > ax) { ax += 1; bx += 1; }
		if ((say || sby) && by > ay) { ay += 1; by += 1; }
	}

	if ((!parallelogram || line) && !fix)
	{
		if (!line && !order_less(bx, by, cx, cy, zb, zc))
		{
			dswap(order1, order2); dswap(bx, cx); dswap(by, cy); dswap(zb, zc);
		}
		if (!order_less(ax, ay, bx, by, za, zb))
		{
			dswap(order0, order1); dswap(ax, bx); dswap(ay, by); dswap(za, zb);
		}
	}
	else if (provoking == 1)
	{
		dswap(order0, order1); dswap(ax, bx); dswap(ay, by); dswap(za, zb);
	}
	else if (provoking == 2)
	{
		dswap(order0, order2); dswap(ax, cx); dswap(ay, cy); dswap(za, zc);
	}

	if (sprite)
	{
		cx = ax; cy = by;
		by = ay;
	}
	else if (line)
	{
		int32_t abx = bx - ax, aby = by - ay;
		if (abs(abx) >= abs(aby))
		{
			int32_t yd = -((abx > 0) - (abx < 0)) * 8;
			if (multisample) yd *= 2;
			cy = ay + yd; ay -= yd; by -= yd;
			if (!multisample) { ay += 1; by += 1; }
			cx = ax;
		}
		else
		{
			int32_t xd = ((aby > 0) - (aby < 0)) * 8;
			if (multisample) xd *= 2;
			cx = ax + xd; ax -= xd; bx -= xd;
			if (!multisample) { ax += 1; bx += 1; }
			cy = ay;
		}
	}

	int32_t abx = bx - ax, aby = by - ay, acx = cx - ax, acy = cy - ay;
	int64_t signed_area = int64_t(aby) * acx - int64_t(abx) * acy;
	if (signed_area == 0)
	{
		out.bb[0] = 0; out.bb[1] = 0; out.bb[2] = -1; out.bb[3] = -1;
		reinterpret_cast<int4 *>(&P.setup[index])[3] = make_int4(0, 0, -1, -1);
		if (sry != 0)
			P.prims[index].state = st | (1u << STATE_BIT_SNAP_ATTRIBUTE);
		return;
	}

	uint32_t area;
	bool flipped = signed_area < 0;
	if (flipped)
	{
		area = uint32_t(0ull - uint64_t(signed_area));
		dswap(abx, acx); dswap(aby, acy);
		dswap(bx, cx); dswap(by, cy);
		dswap(zb, zc);
		dswap(order1, order2);
	}
	else
		area = uint32_t(uint64_t(signed_area));

	int32_t bcx = cx - bx, bcy = cy - by;
	int32_t cax = -acx, cay = -acy;
	int32_t dcdx = aby, dcdy = -abx;
	int32_t dadx = bcy, dady = -bcx;
	int32_t dbdx = cay, dbdy = -cax;
	int64_t const_c = int64_t(-ax) * dcdx - int64_t(ay) * dcdy;
	int64_t const_a = int64_t(-bx) * dadx - int64_t(by) * dady;
	int64_t const_b = int64_t(-cx) * dbdx - int64_t(cy) * dbdy;
	bool tba = tie_break(bcx, bcy), tbb = tie_break(cax, cay), tbc = tie_break(abx, aby);
	int32_t err_a = !tba, err_b = !tbb, err_c = !tbc;
	const_a -= err_a; const_b -= err_b; const_c -= err_c;
	err_a += int32_t(uint64_t(const_a) & 1u);
	err_b += int32_t(uint64_t(const_b) & 1u);
	err_c += int32_t(uint64_t(const_c) & 1u);
	int32_t flip_b = 0, flip_c = 0;
	if (parallelogram)
	{
		int32_t tbo = 1 - int32_t(tbb) - int32_t(tbc);
		flip_b = (tbo + err_b + err_a + 2) >> 1;
		flip_c = (tbo + err_c + err_a + 2) >> 1;
	}

	float inv_area = rcp_fixed(area);
	float inv_area_scaled = fmul(inv_area, 2.0f);
	float error_i = fmul(__int2float_rn(err_b), inv_area);
	float error_j = fmul(__int2float_rn(err_c), inv_area);

	if (sprite) { zb = za; zc = za; }
	else if (line) { zc = za; }
	if (fix || sprite) { order0 = 0; order1 = 1; order2 = 2; }

	pgs_vertex_attribute at0 = P.attr[3 * index + order0];
	pgs_vertex_attribute at1 = P.attr[3 * index + order1];
	pgs_vertex_attribute at2 = {};
	if (!sprite && !line)
		at2 = P.attr[3 * index + order2];

	float s0[4], s1[4], s2[4] = { 0.0f, 0.0f, 0.0f, 0.0f };
	if (perspective)
	{
		s0[0] = at0.s; s0[1] = at0.t; s0[2] = at0.q; s0[3] = at0.fog;
		s1[0] = at1.s; s1[1] = at1.t; s1[2] = at1.q; s1[3] = at1.fog;
		if (!sprite && !line) { s2[0] = at2.s; s2[1] = at2.t; s2[2] = at2.q; s2[3] = at2.fog; }
	}
	else
	{
		s0[0] = fmul(float(at0.u), 0.0625f); s0[1] = fmul(float(at0.v), 0.0625f); s0[2] = at0.q; s0[3] = at0.fog;
		s1[0] = fmul(float(at1.u), 0.0625f); s1[1] = fmul(float(at1.v), 0.0625f); s1[2] = at1.q; s1[3] = at1.fog;
		if (!sprite && !line)
		{
			s2[0] = fmul(float(at2.u), 0.0625f); s2[1] = fmul(float(at2.v), 0.0625f); s2[2] = at2.q; s2[3] = at2.fog;
		}
	}

	if (sprite)
	{
		float o0x = s0[0], o0y = s0[1], o0z = s0[2], o0w = s0[3], o1x = s1[0], o1y = s1[1];
		if (flipped)
		{
			s2[0] = o1x; s2[1] = o0y; s2[2] = o0z; s2[3] = o0w;
			s1[0] = o0x; s1[1] = o1y; s1[2] = o0z; s1[3] = o0w;
		}
		else
		{
			s2[0] = o0x; s2[1] = o1y; s2[2] = o0z; s2[3] = o0w;
			s1[0] = o1x; s1[1] = o0y; s1[2] = o0z; s1[3] = o0w;
		}
	}
	else if (line)
	{
		s2[0] = s0[0]; s2[1] = s0[1]; s2[2] = s0[2]; s2[3] = s0[3];
	}

	if (perspective)
	{
		if (s0[2] < 0.0f)
		{
			s0[0] = -s0[0]; s0[1] = -s0[1]; s1[0] = -s1[0]; s1[1] = -s1[1]; s2[0] = -s2[0]; s2[1] = -s2[1];
		}
		s0[2] = fabsf(s0[2]); s1[2] = fabsf(s1[2]); s2[2] = fabsf(s2[2]);
		uint32_t qexp = (f2u(fmaxf(fmaxf(s0[2], s1[2]), s2[2])) >> 23) & 0xffu;
		s0[2] = u2f(f2u(s0[2]) & ~0xffu);
		s1[2] = u2f(f2u(s1[2]) & ~0xffu);
		s2[2] = u2f(f2u(s2[2]) & ~0xffu);
		uint32_t sexp = (f2u(fmaxf(fmaxf(fabsf(s0[0]), fabsf(s1[0])), fabsf(s2[0]))) >> 23) & 0xffu;
		uint32_t texp = (f2u(fmaxf(fmaxf(fabsf(s0[1]), fabsf(s1[1])), fabsf(s2[1]))) >> 23) & 0xffu;
		uint32_t schop = min(9u + max(sexp, qexp) - sexp, 23u);
		uint32_t tchop = min(9u + max(texp, qexp) - texp, 23u);
		uint32_t smask = ~((1u << schop) - 1u), tmask = ~((1u << tchop) - 1u);
		s0[0] = u2f(f2u(s0[0]) & smask); s1[0] = u2f(f2u(s1[0]) & smask); s2[0] = u2f(f2u(s2[0]) & smask);
		s0[1] = u2f(f2u(s0[1]) & tmask); s1[1] = u2f(f2u(s1[1]) & tmask); s2[1] = u2f(f2u(s2[1]) & tmask);
		bool needs_lod = (pa.tex2 & TEX2_FIXED_LOD_BIT) == 0;
		if (!needs_lod && s0[2] == s1[2] && s0[2] == s2[2])
		{
			float inv_q = rcp_float(s0[2], P.rcp_float_lut);
			s0[0] = fmul(s0[0], inv_q); s0[1] = fmul(s0[1], inv_q);
			s1[0] = fmul(s1[0], inv_q); s1[1] = fmul(s1[1], inv_q);
			s2[0] = fmul(s2[0], inv_q); s2[1] = fmul(s2[1], inv_q);
			s0[2] = 1.0f; s1[2] = 1.0f; s2[2] = 1.0f;
		}
	}

	float di[4], dj[4];
	#pragma unroll
	for (int k = 0; k < 4; k++)
	{
		di[k] = fix ? 0.0f : fsub(s1[k], s0[k]);
		dj[k] = fix ? 0.0f : fsub(s2[k], s0[k]);
		ta.stqf0[k] = s0[k];
		ta.stqf1[k] = di[k];
		ta.stqf2[k] = dj[k];
	}
	if (iip && !sprite)
	{
		uint32_t r0 = at0.rgba, r1 = at1.rgba, r2 = at2.rgba;
		if (fix) r1 = r0;
		if (fix || line) r2 = r0;
		set_color_terms(P, ta, r0, r1, r2);
	}
	else
	{
		uint32_t flat = P.attr[3 * index].rgba;
		set_color_terms(P, ta, flat, flat, flat);
	}

	int32_t pa0 = dadx, pa1 = dady, pa2 = int32_t(uint32_t(uint64_t(const_a) >> 1));
	int32_t pb0 = dbdx, pb1 = dbdy, pb2 = int32_t(uint32_t(uint64_t(const_b) >> 1));
	int32_t pc0 = dcdx, pc1 = dcdy, pc2 = int32_t(uint32_t(uint64_t(const_c) >> 1));
	uint32_t axw = (uint32_t(pa0) << 6) & ~1u;
	axw |= uint32_t(parallelogram);
	axw = (axw & ~(3u << 2)) | ((uint32_t(flip_b) & 3u) << 2);
	axw = (axw & ~(3u << 4)) | ((uint32_t(flip_c) & 3u) << 4);

	int32_t dx = parallelogram ? (bx + cx - ax) : cx;
	int32_t dy = parallelogram ? (by + cy - ay) : cy;

	int32_t di_r = 0, dj_r = 0;
	if (sprite)
	{
		int32_t xd = dx - ax, yd = dy - ay;
		if (xd > 0 && (xd & (xd - 1)) != 0) { di_r += pb0; dj_r += pc0; }
		if (yd > 0 && (yd & (yd - 1)) != 0) { di_r += pb1; dj_r += pc1; }
	}
	else if (parallelogram && !perspective)
	{
		bool nearest = (pa.tex & TEX_SAMPLER_MAG_LINEAR_BIT) == 0;
		bool npot_area = (area & (area - 1)) != 0;
		if (nearest && npot_area)
		{
			int32_t d0x = int32_t(at0.u) - ax, d0y = int32_t(at0.v) - ay;
			int32_t d1x = int32_t(at1.u) - bx, d1y = int32_t(at1.v) - by;
			int32_t d2x = int32_t(at2.u) - cx, d2y = int32_t(at2.v) - cy;
			if (d0x == d1x && d0y == d1y && d0x == d2x && d0y == d2y)
			{
				bool mis_x = (min(ax, dx) & 15) != 0, mis_y = (min(ay, dy) & 15) != 0;
				float dudx = fadd(fmul(di[0], float(pb0)), fmul(dj[0], float(pc0)));
				float dvdx = fadd(fmul(di[1], float(pb0)), fmul(dj[1], float(pc0)));
				float dudy = fadd(fmul(di[0], float(pb1)), fmul(dj[0], float(pc1)));
				float dvdy = fadd(fmul(di[1], float(pb1)), fmul(dj[1], float(pc1)));
				bool adj_x = mis_x && ((dudx > 0.0f && dvdx == 0.0f) || (dvdx > 0.0f && dudx == 0.0f));
				bool adj_y = mis_y && ((dudy > 0.0f && dvdy == 0.0f) || (dvdy > 0.0f && dudy == 0.0f));
				if (adj_x) { di_r -= pb0; dj_r -= pc0; }
				if (adj_y) { di_r -= pb1; dj_r -= pc1; }
			}
		}
	}
	float eighth = fmul(0.125f, inv_area_scaled);
	error_i = fadd(error_i, fmul(__int2float_rn(di_r), eighth));
	error_j = fadd(error_j, fmul(__int2float_rn(dj_r), eighth));

	out.a[0] = int32_t(axw); out.a[1] = pa1; out.a[2] = pa2;
	out.b[0] = pb0; out.b[1] = pb1; out.b[2] = pb2;
	out.c[0] = pc0; out.c[1] = pc1; out.c[2] = pc2;
	out.inv_area = inv_area_scaled;
	out.error_i = error_i;
	out.error_j = error_j;
	out.z[0] = za;
	out.z[1] = f2u(__uint2float_rn(zb - za));
	out.z[2] = f2u(__uint2float_rn(zc - za));
	out.z[3] = 0;

	int32_t lox = min(min(ax, bx), min(cx, dx)), loy = min(min(ay, by), min(cy, dy));
	int32_t hix = max(max(ax, bx), max(cx, dx)), hiy = max(max(ay, by), max(cy, dy));
	lox = (lox + (15 >> sry)) >> 4;
	loy = (loy + (15 >> sry)) >> 4;
	hix = (hix - 1) >> 4;
	hiy = (hiy - 1) >> 4;
	if (multisample && !line) { lox -= 1; loy -= 1; hix += 1; hiy += 1; }
	out.bb[0] = max(lox, int32_t(pa.bb[0]));
	out.bb[1] = max(loy, int32_t(pa.bb[1]));
	out.bb[2] = min(hix, int32_t(pa.bb[2]));
	out.bb[3] = min(hiy, int32_t(pa.bb[3]));

	uint32_t tex = pa.tex;
	if (sprite && !perspective)
	{
		int32_t u0x = int32_t(at0.u) - ax, u0y = int32_t(at0.v) - ay;
		int32_t u1x = int32_t(at1.u) - dx, u1y = int32_t(at1.v) - dy;
		int32_t mnx = min(u0x, u1x), mny = min(u0y, u1y), mxx = max(u0x, u1x), mxy = max(u0y, u1y);
		bool csx = (mnx & 15) == 8, csy = (mny & 15) == 8;
		bool nsx = (mxx & 15) == 9, nsy = (mxy & 15) == 9;
		int32_t ddx = abs(dx - ax), ddy = abs(dy - ay);
		nsx = nsx && (ddx & (ddx - 1)) != 0;
		nsy = nsy && (ddy & (ddy - 1)) != 0;
		bool no_interp = (mxx - mnx) <= 1 && (mxy - mny) <= 1;
		if ((nsx || csx) && (nsy || csy) && no_interp)
			tex &= ~TEX_SAMPLER_MAG_LINEAR_BIT;
	}

	uint32_t new_state = st;
	if (pa.fbmsk != opaque_fbmask && (new_state & (1u << STATE_BIT_OPAQUE)))
		new_state &= ~(1u << STATE_BIT_OPAQUE);

	// Super-sampled textures (triangle_setup.comp:677-825): nearest blits map
	// sample to sample, nearest downsamples and blur kernels fall back to the
	// single-sampled layer, linear upsamples read the resolved layer (with
	// FORCE_LINEAR_SUPER_SAMPLE, for field rendering, blur kernels read the
	// resolved layer linearly and linear downsamples and upsamples stay per
	// sample); what stays per-sample interpolates per sample around the
	// single-sampled mean position.
	if (sry != 0 && (tex & (TEX_PER_SAMPLE_BIT | TEX_SAMPLE_MAPPING_BIT)) == TEX_PER_SAMPLE_BIT)
	{
		const int32_t udx = abs(int32_t(at1.u) - int32_t(at0.u)), udy = abs(int32_t(at1.v) - int32_t(at0.v));
		const int32_t ddx = abs(dx - ax), ddy = abs(dy - ay);
		if ((tex & TEX_SAMPLER_MAG_LINEAR_BIT) == 0)
		{
			if (perspective)
				tex |= TEX_SAMPLE_MAPPING_BIT;
			else if (udx > ddx + 1 || udy > ddy + 1)
				tex &= ~TEX_PER_SAMPLE_BIT;
			else if (udx >= ddx - 16 || udy >= ddy - 16)
			{
				const uint32_t blend = P.states[min(st & STATE_INDEX_MASK, P.num_states - 1u)].blend_mode;
				const uint32_t inst = (st >> STATE_VERTEX_RENDER_PASS_INSTANCE_OFFSET) & 7u;
				const bool blur = ((P.rp_is_blur_mask >> inst) & 1u) && (blend & BLEND_MODE_ABE_BIT) &&
				                  !(st & (1u << STATE_BIT_Z_TEST)) &&
				                  ((blend >> BLEND_MODE_A_MODE_OFFSET) & 3u) == BLEND_RGB_SOURCE &&
				                  ((blend >> BLEND_MODE_B_MODE_OFFSET) & 3u) == BLEND_RGB_ZERO &&
				                  ((blend >> BLEND_MODE_D_MODE_OFFSET) & 3u) == BLEND_RGB_DEST;
				if (blur && P.force_linear_ss)
				{
					// Field rendering keeps blur kernels per sample: the
					// resolved layer, filtered linearly, with the mean sample
					// position moved to the texel centre
					// (triangle_setup.comp:729-746).
					tex |= TEX_SAMPLE_RESOLVED_BIT | TEX_SAMPLER_MAG_LINEAR_BIT;
					const int32_t avg_u = (int32_t(at0.u) + int32_t(at1.u)) >> 1;
					const int32_t avg_v = (int32_t(at0.v) + int32_t(at1.v)) >> 1;
					const int32_t ph_x = (avg_u - ((dx + ax) >> 1)) & 15, ph_y = (avg_v - ((dy + ay) >> 1)) & 15;
					ta.stqf0[0] = fadd(ta.stqf0[0], fsub(0.5f, fmul(__int2float_rn(ph_x), 0.0625f)));
					ta.stqf0[1] = fadd(ta.stqf0[1], fsub(0.5f, fmul(__int2float_rn(ph_y), 0.0625f)));
				}
				else if (blur)
					tex &= ~TEX_PER_SAMPLE_BIT;
				else
					tex |= TEX_SAMPLE_MAPPING_BIT;
			}
		}
		else if (!perspective)
		{
			if (udx > ddx + 1 && udy > ddy + 1)
			{
				if (!P.force_linear_ss)
					tex &= ~TEX_PER_SAMPLE_BIT;
			}
			else if (ddx >= 2 * udx && ddy >= 2 * udy)
			{
				if (!P.force_linear_ss)
					tex |= TEX_SAMPLE_RESOLVED_BIT;
			}
		}
		if ((tex & (TEX_PER_SAMPLE_BIT | TEX_SAMPLE_MAPPING_BIT)) == TEX_PER_SAMPLE_BIT)
		{
			new_state &= ~(1u << STATE_BIT_SNAP_ATTRIBUTE);
			const float corner = fmul(8.0f, average_sampling_offset(P.setup_rate_x_log2, P.setup_rate_y_log2));
			const float di_dcorner = fmul(__int2float_rn(pb0 + pb1), corner);
			const float dj_dcorner = fmul(__int2float_rn(pc0 + pc1), corner);
			out.error_i = fsub(out.error_i, fmul(di_dcorner, inv_area_scaled));
			out.error_j = fsub(out.error_j, fmul(dj_dcorner, inv_area_scaled));
		}
	}

	if (sry != 0 && !sprite)
	{
		bool per_sample = multisample;
		if (!per_sample && perspective)
			per_sample = di[2] != 0.0f || dj[2] != 0.0f;
		if (!per_sample)
			per_sample = za != zb || zb != zc;
		if (!per_sample)
		{
			// Flat primitive: snap attributes and register its depth bucket
			// for the single-sample heuristic (triangle_setup.comp:826-871).
			if (!line)
				new_state |= 1u << STATE_BIT_SNAP_ATTRIBUTE;
			uint32_t inst = (st >> STATE_VERTEX_RENDER_PASS_INSTANCE_OFFSET) & 7u;
			uint32_t z_shift = ((P.packed_z_shift >> (4 * inst)) & 15u) * 8u;
			uint32_t bucket = min(255u, z_shift >= 32 ? 0u : za >> z_shift);
			uint32_t old = atomicOr(&P.heuristic->active[bucket >> 5], 1u << (bucket & 31));
			if (((old >> (bucket & 31)) & 1u) == 0)
			{
				uint32_t slot = atomicAdd(&P.heuristic->bucket_count, 1u);
				P.heuristic->bucket[slot] = bucket;
			}
		}
	}

	P.setup[index] = out;
	P.tattr[index] = ta;
	P.prims[index].state = new_state;
	P.prims[index].tex = tex;
}

// ---------------------------------------------------------------------------
// Single-sample heuristic (single_sample_heuristic.comp:148-291): for every
// depth bucket that holds a flat primitive, decide which flat primitives are
// UI elements to rasterise single-sampled (SNAP_RASTER) and which sit inside
// the 3D depth range and go back to full SSAA (SNAP_ATTRIBUTE cleared).
// One CTA per (bucket, instance); 3 x 64K-bit masks in shared memory.
// Decisions go to P.heuristic_action so that every bucket reads the states
// triangle setup wrote, whatever order the CTAs run in.

__device__ __forceinline__ uint32_t heuristic_hash_vertex(const pgs_vertex_position &v)
{
	// Three rounds of ((s >> 8) ^ s.yzx) * 1103515245 (:86-94).
	uint32_t x = uint32_t(v.x), y = uint32_t(v.y), z = v.z;
	#pragma unroll
	for (int r = 0; r < 3; r++)
	{
		uint32_t nx = ((x >> 8) ^ y) * 1103515245u;
		uint32_t ny = ((y >> 8) ^ z) * 1103515245u;
		uint32_t nz = ((z >> 8) ^ x) * 1103515245u;
		x = nx; y = ny; z = nz;
	}
	return x >> 16;
}

constexpr uint32_t HEURISTIC_MASK_WORDS = 65536 / 32;

__global__ void __launch_bounds__(1024) single_sample_heuristic_kernel(PassParams P, HeuristicParams H)
{
	const uint32_t inst = blockIdx.y;
	if (((H.instance_mask >> inst) & 1u) == 0)
		return;
	if (blockIdx.x >= P.heuristic->bucket_count)
		return;

	__shared__ uint32_t full3d[HEURISTIC_MASK_WORDS];
	__shared__ uint32_t candidate[HEURISTIC_MASK_WORDS];
	__shared__ uint32_t shared_vertex[HEURISTIC_MASK_WORDS];
	__shared__ uint32_t any_full3d, min_z, max_z;

	const uint32_t tid = threadIdx.x, nthreads = blockDim.x;
	for (uint32_t i = tid; i < HEURISTIC_MASK_WORDS; i += nthreads)
	{
		full3d[i] = 0;
		candidate[i] = 0;
		shared_vertex[i] = 0;
	}
	if (tid == 0)
	{
		any_full3d = 0;
		min_z = ~0u;
		max_z = 0;
	}
	__syncthreads();

	const uint32_t z_shift = H.z_shift[inst], z_max = H.z_max[inst];
	uint32_t zlo = P.heuristic->bucket[blockIdx.x];
	uint32_t zhi = ((zlo + 1) << H.z_shift_bucket[inst]) - 1;
	zlo <<= H.z_shift_bucket[inst];

	const uint32_t SA = 1u << STATE_BIT_SNAP_ATTRIBUTE, SR = 1u << STATE_BIT_SNAP_RASTER;
	const uint32_t LINE = 1u << STATE_BIT_LINE;
	const uint32_t NO_FULL_3D = (1u << STATE_BIT_SPRITE) | LINE | SA;
	const uint32_t n = P.num_prims;
	auto inst_of = [](uint32_t st) { return (st >> STATE_VERTEX_RENDER_PASS_INSTANCE_OFFSET) & 7u; };
	auto snap = [&](uint32_t z) { return min(z_max, z) >> z_shift; };

	// Pass 1: depth values used by 3D primitives, and flat candidates.
	uint32_t lmin = ~0u, lmax = 0, lany = 0;
	for (uint32_t i = tid; i < n; i += nthreads)
	{
		uint32_t st = P.prims[i].state;
		if (inst_of(st) != inst)
			continue;
		if ((st & NO_FULL_3D) == 0)
		{
			#pragma unroll
			for (int k = 0; k < 3; k++)
			{
				uint32_t z = P.pos[3 * i + k].z;
				lmin = min(lmin, z);
				lmax = max(lmax, z);
				uint32_t s = snap(z);
				if (s >= zlo && s <= zhi)
					atomicOr(&full3d[(s - zlo) >> 5], 1u << ((s - zlo) & 31));
			}
			lany = 1;
		}
		else if ((st & (SA | SR)) == SA || (st & LINE) != 0)
		{
			uint32_t s = snap(P.pos[3 * i].z);
			if (s >= zlo && s <= zhi)
				atomicOr(&candidate[(s - zlo) >> 5], 1u << ((s - zlo) & 31));
		}
	}
	lmin = __reduce_min_sync(0xffffffffu, lmin);
	lmax = __reduce_max_sync(0xffffffffu, lmax);
	lany = __reduce_or_sync(0xffffffffu, lany);
	if ((tid & 31) == 0)
	{
		atomicMin(&min_z, lmin);
		atomicMax(&max_z, lmax);
		if (lany)
			any_full3d = 1;
	}
	__syncthreads();

	// Pass 2: hash the vertices of 3D primitives whose depth is a candidate.
	for (uint32_t i = tid; i < n; i += nthreads)
	{
		uint32_t st = P.prims[i].state;
		if (inst_of(st) != inst || (st & NO_FULL_3D) != 0)
			continue;
		#pragma unroll
		for (int k = 0; k < 3; k++)
		{
			pgs_vertex_position v = P.pos[3 * i + k];
			uint32_t s = snap(v.z);
			if (s >= zlo && s <= zhi && ((candidate[(s - zlo) >> 5] >> ((s - zlo) & 31)) & 1u))
			{
				uint32_t h = heuristic_hash_vertex(v);
				atomicOr(&shared_vertex[h >> 5], 1u << (h & 31));
			}
		}
	}
	__syncthreads();

	// Pass 3: a flat candidate that shares a vertex with a 3D primitive at a
	// depth the 3D geometry uses keeps its depth out of demotion.
	for (uint32_t i = tid; i < n; i += nthreads)
	{
		uint32_t st = P.prims[i].state;
		if (inst_of(st) != inst || (st & (SA | SR)) != SA)
			continue;
		uint32_t s = snap(P.pos[3 * i].z);
		if (s < zlo || s > zhi)
			continue;
		uint32_t o = s - zlo;
		if (((full3d[o >> 5] >> (o & 31)) & 1u) == 0)
			continue;
		bool conflict = false;
		#pragma unroll
		for (int k = 0; k < 3; k++)
		{
			uint32_t h = heuristic_hash_vertex(P.pos[3 * i + k]);
			conflict |= ((shared_vertex[h >> 5] >> (h & 31)) & 1u) != 0;
		}
		if (conflict)
			atomicAnd(&candidate[o >> 5], ~(1u << (o & 31)));
	}
	__syncthreads();

	// Pass 4: decisions.
	const bool force_single_sample = any_full3d == 0;
	const uint32_t zmin3d = min_z, zmax3d = max_z;
	for (uint32_t i = tid; i < n; i += nthreads)
	{
		uint32_t z = P.pos[3 * i].z;
		uint32_t s = snap(z);
		if (s < zlo || s > zhi)
			continue;
		uint32_t st = P.prims[i].state;
		if (inst_of(st) != inst)
			continue;
		bool tri_candidate = (st & (SA | SR)) == SA;
		bool line_candidate = force_single_sample && (st & LINE) != 0;
		if (!tri_candidate && !line_candidate)
			continue;
		uint32_t o = s - zlo;
		if ((candidate[o >> 5] >> (o & 31)) & 1u)
			P.heuristic_action[i] = HEURISTIC_SET_SNAP_RASTER;
		else if ((st & ((1u << STATE_BIT_Z_TEST) | (1u << STATE_BIT_Z_WRITE))) != 0 && z > zmin3d && z < zmax3d)
			P.heuristic_action[i] = HEURISTIC_CLEAR_SNAP_ATTRIBUTE;
	}
}

// Applies and clears the heuristic's decisions.
__global__ void __launch_bounds__(256) heuristic_apply_kernel(PassParams P)
{
	uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
	if (i >= P.num_prims)
		return;
	uint8_t a = P.heuristic_action[i];
	if (a == 0)
		return;
	uint32_t st = P.prims[i].state;
	if (a == HEURISTIC_SET_SNAP_RASTER)
		st |= 1u << STATE_BIT_SNAP_RASTER;
	else
		st &= ~(1u << STATE_BIT_SNAP_ATTRIBUTE);
	P.prims[i].state = st;
	P.heuristic_action[i] = 0;
}

// ---------------------------------------------------------------------------
// Conservative tile test (intersect.h:24-81).
__device__ __forceinline__ bool intersects_tile(const PrimSetup &s, int32_t lo0, int32_t lo1, int32_t hi0, int32_t hi1,
                                                bool ms_tri)
{
	int32_t l0 = max(s.bb[0], lo0), l1 = max(s.bb[1], lo1);
	int32_t h0 = min(s.bb[2], hi0), h1 = min(s.bb[3], hi1);
	if (h0 < l0 || h1 < l1)
		return false;
	int32_t axw = s.a[0];
	bool par = (axw & 1) != 0;
	int32_t off_b = int32_t((uint32_t(axw) >> 2) & 3u) - 1;
	int32_t off_c = int32_t((uint32_t(axw) >> 4) & 3u) - 1;
	int32_t A[3] = { axw >> 6, s.a[1], s.a[2] };
	l0 <<= 3; l1 <<= 3;
	h0 = (h0 << 3) | 7; h1 = (h1 << 3) | 7;
	int32_t da = idot3(A, A[0] >= 0 ? h0 : l0, A[1] >= 0 ? h1 : l1);
	int32_t db = idot3(s.b, s.b[0] >= 0 ? h0 : l0, s.b[1] >= 0 ? h1 : l1);
	int32_t dc = idot3(s.c, s.c[0] >= 0 ? h0 : l0, s.c[1] >= 0 ? h1 : l1);
	if (ms_tri && !par)
	{
		da += 8 * max(abs(A[0]), abs(A[1]));
		db += 8 * max(abs(s.b[0]), abs(s.b[1]));
		dc += 8 * max(abs(s.c[0]), abs(s.c[1]));
	}
	bool ok = da >= 0 && db >= 0 && dc >= 0;
	if (par && !ok)
	{
		da = idot3(A, A[0] >= 0 ? h0 : l0, A[1] >= 0 ? h1 : l1);
		db = idot3(s.b, -s.c[0] >= 0 ? h0 : l0, -s.c[1] >= 0 ? h1 : l1);
		dc = idot3(s.c, -s.b[0] >= 0 ? h0 : l0, -s.b[1] >= 0 ? h1 : l1);
		db += da + off_b;
		dc += da + off_c;
		da = idot3(A, A[0] >= 0 ? l0 : h0, A[1] >= 0 ? l1 : h1);
		ok = (-1 >= da) && db >= 0 && dc >= 0;
	}
	return ok;
}

// ---------------------------------------------------------------------------
// K2: binning.  Coarse tiles (2^tile_size_log2 pixels) carry the reference's
// membership test and super-sampling flags (binning.comp:74-125); shading
// lists are kept per 8x8 sub-tile as bitmasks over the pass's primitive range
// so that ascending primitive order needs no sort.  A summary bitmask marks
// non-empty mask words.  A CTA takes 32 primitives (one mask word): each of
// its BIN_GROUP_WARPS warps loads all 32, warp 0 marks the coarse tiles, and
// the warps share the (primitive, sub-tile) tests, so that the dependent
// loads and shuffles of one batch overlap those of the others.
constexpr uint32_t BIN_GROUP_WARPS = 4;

__global__ void __launch_bounds__(32 * BIN_GROUP_WARPS) bin_kernel(PassParams P, DevInstance I, uint32_t *sub_masks,
                                                                   uint32_t *sub_summary, uint32_t *tile_flags)
{
	const unsigned full = 0xffffffffu;
	const uint32_t lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
	const uint32_t local = blockIdx.x * 32u + lane;
	const uint32_t p = I.prim_lo + local;
	bool live = local < I.prim_count;
	pgs_primitive_attribute pa = {};
	PrimSetup s = {};
	if (live)
	{
		pa = P.prims[p];
		live = ((pa.state >> STATE_VERTEX_RENDER_PASS_INSTANCE_OFFSET) & 7u) == I.instance;
	}
	if (live)
	{
		s = P.setup[p];
		live = !(s.bb[2] < s.bb[0] || s.bb[3] < s.bb[1]);
	}

	const int ts = int(P.tile_size_log2);
	const bool ms_tri = ((pa.state >> STATE_BIT_MULTISAMPLE) & 1) && !((pa.state >> STATE_BIT_LINE) & 1);
	// Coarse tiles: membership and super-sampling flags, one primitive per
	// thread of warp 0.
	if (warp == 0 && live)
	{
		int32_t tx0 = max((s.bb[0] - I.base_x) >> ts, 0), ty0 = max((s.bb[1] - I.base_y) >> ts, 0);
		int32_t tx1 = min((s.bb[2] - I.base_x) >> ts, int32_t(I.tiles_w) - 1);
		int32_t ty1 = min((s.bb[3] - I.base_y) >> ts, int32_t(I.tiles_h) - 1);
		uint32_t flags = TILE_NONEMPTY;
		if (I.rate_y_log2 != 0)
		{
			const uint32_t full_mask = (1u << STATE_BIT_SNAP_RASTER) | (1u << STATE_BIT_Z_TEST) | (1u << STATE_BIT_OPAQUE);
			const uint32_t color_mask = (1u << STATE_BIT_SNAP_RASTER) | (1u << STATE_BIT_OPAQUE);
			if ((pa.state & full_mask) != color_mask) flags |= TILE_REQ_SS_ZW;
			if ((pa.state & color_mask) != color_mask) flags |= TILE_REQ_SS;
			if (pa.state & (1u << STATE_BIT_Z_WRITE)) flags |= TILE_HAS_ZW;
			if (pa.tex & TEX_PER_SAMPLE_BIT) flags |= TILE_REQ_SS;
		}
		for (int32_t ty = ty0; ty <= ty1; ty++)
			for (int32_t tx = tx0; tx <= tx1; tx++)
			{
				int32_t lo0 = I.base_x + (tx << ts), lo1 = I.base_y + (ty << ts);
				if (!intersects_tile(s, lo0, lo1, lo0 + (1 << ts) - 1, lo1 + (1 << ts) - 1, ms_tri))
					continue;
				uint32_t tile = uint32_t(ty) * I.tiles_w + uint32_t(tx);
				atomicOr(&tile_flags[tile], flags);
				if (I.blend_demote)
					atomicAdd(&tile_flags[tile], 1u << TILE_COUNT_SHIFT);
			}
	}

	// 8x8 sub-tiles: the warp's (primitive, sub-tile) candidates are dealt out
	// to its lanes 32 at a time, so one large primitive does not hold the warp.
	// A sub-tile that passes the test lies in a coarse tile that passes it
	// (the test is monotonic in the rectangle), so testing the sub-tiles of the
	// primitive's box inside the instance is the same as testing those of its
	// member coarse tiles.
	int32_t gx0 = 0, gy0 = 0, gw = 0, gh = 0;
	if (live)
	{
		const int32_t xmax = I.base_x + int32_t(I.tiles_w << ts) - 1, ymax = I.base_y + int32_t(I.tiles_h << ts) - 1;
		const int32_t x0 = max(s.bb[0], I.base_x), y0 = max(s.bb[1], I.base_y);
		const int32_t x1 = min(s.bb[2], xmax), y1 = min(s.bb[3], ymax);
		if (x1 >= x0 && y1 >= y0)
		{
			gx0 = (x0 - I.base_x) >> 3;
			gy0 = (y0 - I.base_y) >> 3;
			gw = ((x1 - I.base_x) >> 3) - gx0 + 1;
			gh = ((y1 - I.base_y) >> 3) - gy0 + 1;
		}
	}
	const uint32_t count = uint32_t(gw * gh);
	uint32_t incl = count;
	#pragma unroll
	for (int o = 1; o < 32; o <<= 1)
	{
		const uint32_t y = __shfl_up_sync(full, incl, o);
		if (lane >= uint32_t(o))
			incl += y;
	}
	const uint32_t total = __shfl_sync(full, incl, 31);
	const uint32_t warp_first = blockIdx.x * 32u;
	for (uint32_t base = warp * 32u; base < total; base += 32u * BIN_GROUP_WARPS)
	{
		const uint32_t j = base + lane;
		// Owner: the first lane whose inclusive count exceeds j.
		uint32_t lo = 0, hi = 31;
		#pragma unroll
		for (int it = 0; it < 5; it++)
		{
			const uint32_t mid = (lo + hi) >> 1;
			const uint32_t v = __shfl_sync(full, incl, int(mid));
			if (v > j)
				hi = mid;
			else
				lo = mid + 1u;
		}
		const uint32_t o = lo;
		const uint32_t o_incl = __shfl_sync(full, incl, int(o)), o_count = __shfl_sync(full, count, int(o));
		const int32_t o_gx0 = __shfl_sync(full, gx0, int(o)), o_gy0 = __shfl_sync(full, gy0, int(o));
		const int32_t o_gw = __shfl_sync(full, gw, int(o));
		const bool o_ms = __shfl_sync(full, ms_tri ? 1 : 0, int(o)) != 0;
		if (j >= total)
			continue;
		const uint32_t k = j - (o_incl - o_count);
		const int32_t gx = o_gx0 + int32_t(k % uint32_t(o_gw)), gy = o_gy0 + int32_t(k / uint32_t(o_gw));
		const uint32_t o_local = warp_first + o;
		const PrimSetup &os = P.setup[I.prim_lo + o_local];
		const int32_t sx = I.base_x + (gx << 3), sy = I.base_y + (gy << 3);
		if (!intersects_tile(os, sx, sy, sx + 7, sy + 7, o_ms))
			continue;
		// Results unused: both compile to fire-and-forget reductions.
		const uint32_t word = o_local >> 5, bit = 1u << (o_local & 31u);
		const uint32_t sword = word >> 5, sbit = 1u << (word & 31u);
		const size_t sub = size_t(gy) * I.sub_w + size_t(gx);
		atomicOr(&sub_masks[sub * I.mask_words + word], bit);
		atomicOr(&sub_summary[sub * I.summary_words + sword], sbit);
	}
}

// ---------------------------------------------------------------------------
// K5: texture decode.  One thread per texel of every texture of the pass.
__global__ void __launch_bounds__(256) texture_decode_kernel(PassParams P);

// ---------------------------------------------------------------------------
// K3: shading.
// A pending or candidate shade of one sample.  Only what changes per sample
// is kept; the state index, Z comparison, perspective and AA1 flags are
// read back from the primitive's state word when needed.
struct Request
{
	int coverage;
	bool z_test, z_write;
	uint32_t z;
	float i, j;
};

// unpackUnorm4x8 channel: float(c) / 255 correctly rounded.  The 256 values are
// computed on the host with IEEE division and read from a table.
__device__ __forceinline__ float unorm8(uint32_t c, int ch) { return __fdiv_rn(float((c >> (8 * ch)) & 0xffu), 255.0f); }

__device__ __forceinline__ uint32_t pack_unorm(float r, float g, float b, float a)
{
	float v[4] = { r, g, b, a };
	uint32_t out = 0;
	#pragma unroll
	for (int k = 0; k < 4; k++)
	{
		float x = fminf(fmaxf(v[k], 0.0f), 1.0f);
		out |= uint32_t(rintf(fmul(x, 255.0f))) << (8 * k);
	}
	return out;
}

__device__ __forceinline__ uint32_t expand16(uint32_t c)
{
	uint32_t r = (c & 0x1fu) << 3, g = ((c >> 5) & 0x1fu) << 3, b = ((c >> 10) & 0x1fu) << 3;
	return r | (g << 8) | (b << 16) | ((c & 0x8000u) ? 0x80000000u : 0u);
}

struct ShadeCtx
{
	const PassParams *P;
	const DevInstance *I;
	bool ss;
	int dim;          // sampling rate y log2 when super-sampled, else 0
	int32_t snap_mask_x, snap_mask_y;
	bool zs;
	uint32_t fb_psm, zb_psm;
	uint32_t sample; // sample index of the thread in a super-sampled tile, else 0
};

__device__ __forceinline__ uint32_t clut_color(const PassParams &P, const pgs_texture_desc &t, uint32_t index)
{
	uint32_t bi = t.csa * 16u + index;
	bool c16 = t.cpsm == PSMCT16 || t.cpsm == PSMCT16S;
	if (t.psm == PSMT8 || t.psm == PSMT8H)
	{
		uint32_t bank = min(bi >> 4, c16 ? 31u : 15u);
		bi = bank * 16u + (bi & 15u);
	}
	bi = min(bi, c16 ? 511u : 255u);
	const uint16_t *cl = P.clut + size_t(t.clut_instance % PGS_CLUT_INSTANCES) * 512u;
	if (c16)
		return rgba16_to_rgba32(__ldg(cl + bi), t.aem, t.ta0, t.ta1);
	return uint32_t(__ldg(cl + bi)) | (uint32_t(__ldg(cl + bi + 256u)) << 16);
}

// The VRAM a texture of the pass decodes from: a snapshot taken before a
// transfer overwrote its source, or VRAM as the pass begins.
__device__ __forceinline__ const uint8_t *texture_source(const PassParams &P, uint32_t tex)
{
	for (uint32_t k = 0; k < P.num_snaps; k++)
		if (tex < P.snap_limit[k])
			return P.snap_vram[k];
	return P.vram;
}

__device__ __forceinline__ uint32_t fetch_texel(const PassParams &P, const uint8_t *v, const pgs_texture_desc &t,
                                                uint32_t tbp, uint32_t tbw, int32_t x, int32_t y)
{
	uint32_t a = swizzle_address(uint32_t(x), uint32_t(y), tbp, tbw, t.psm);
	switch (t.psm)
	{
	case PSMCT24: case PSMZ24:
		return rgb24_to_rgba32(__ldg(reinterpret_cast<const uint32_t *>(v) + a), t.aem, t.ta0);
	case PSMCT16: case PSMCT16S: case PSMZ16: case PSMZ16S:
		return rgba16_to_rgba32(__ldg(reinterpret_cast<const uint16_t *>(v) + a), t.aem, t.ta0, t.ta1);
	case PSMT8: return clut_color(P, t, __ldg(v + a));
	case PSMT8H: return clut_color(P, t, __ldg(v + 4u * a + 3u));
	case PSMT4: return clut_color(P, t, (uint32_t(__ldg(v + (a >> 1))) >> ((a & 1u) * 4u)) & 15u);
	case PSMT4HL: return clut_color(P, t, (__ldg(reinterpret_cast<const uint32_t *>(v) + a) >> 24) & 15u);
	case PSMT4HH: return clut_color(P, t, __ldg(reinterpret_cast<const uint32_t *>(v) + a) >> 28);
	default: return __ldg(reinterpret_cast<const uint32_t *>(v) + a);
	}
}

// Texel of sample `s` of a super-sampled texture: the single-sampled texel
// unless the reference plane marks it super-sampled (upload.comp
// SUPER_SAMPLED, :131-220; 24-bit formats merge by the reference bits).
__device__ __forceinline__ uint32_t fetch_texel_sample(const PassParams &P, const uint8_t *v, const pgs_texture_desc &t,
                                                       int32_t x, int32_t y, uint32_t s)
{
	const uint32_t a = swizzle_address(uint32_t(x), uint32_t(y), t.tbp0, t.tbw, t.psm);
	const uint32_t *v32 = reinterpret_cast<const uint32_t *>(v);
	const uint16_t *v16 = reinterpret_cast<const uint16_t *>(v);
	const uint32_t V32 = VRAM_SIZE / 4, V16 = VRAM_SIZE / 2, V8 = VRAM_SIZE;
	switch (t.psm)
	{
	case PSMCT24: case PSMZ24:
	{
		uint32_t col = __ldg(v32 + a), ref = __ldg(v32 + a + V32);
		if (ref != 0u)
			col = (__ldg(v32 + a + (2u + s) * V32) & ref) | (col & ~ref);
		return rgb24_to_rgba32(col, t.aem, t.ta0);
	}
	case PSMCT16: case PSMCT16S: case PSMZ16: case PSMZ16S:
	{
		uint32_t col = __ldg(v16 + a);
		if (__ldg(v16 + a + V16) == 0xffffu)
			col = __ldg(v16 + a + (2u + s) * V16);
		return rgba16_to_rgba32(col, t.aem, t.ta0, t.ta1);
	}
	case PSMT8:
	{
		uint32_t idx = __ldg(v + a);
		if (__ldg(v + a + V8) == 0xffu)
			idx = __ldg(v + a + (2u + s) * V8);
		return clut_color(P, t, idx);
	}
	case PSMT8H:
	{
		const uint32_t a8 = 4u * a + 3u;
		uint32_t idx = __ldg(v + a8);
		if (__ldg(v + a8 + V8) == 0xffu)
			idx = __ldg(v + a8 + (2u + s) * V8);
		return clut_color(P, t, idx);
	}
	default:
	{
		uint32_t col = __ldg(v32 + a);
		if (__ldg(v32 + a + V32) == 0xffffffffu)
			col = __ldg(v32 + a + (2u + s) * V32);
		return col;
	}
	}
}

__device__ __forceinline__ void effective_wrap(pgs_texture_desc &t, uint32_t tex_word)
{
	if (t.wms < WRAP_REGION_CLAMP)
		t.wms = (tex_word & TEX_SAMPLER_CLAMP_S_BIT) ? WRAP_CLAMP : WRAP_REPEAT;
	if (t.wmt < WRAP_REGION_CLAMP)
		t.wmt = (tex_word & TEX_SAMPLER_CLAMP_T_BIT) ? WRAP_CLAMP : WRAP_REPEAT;
}

// A wrap mode as (v & and_mask | or_mask) clamped to [lo, hi]: REPEAT masks,
// CLAMP and REGION_CLAMP clamp, REGION_REPEAT masks with MINU and ors MAXU.
struct WrapAxis
{
	int32_t and_mask, or_mask, lo, hi;
};

__device__ __forceinline__ WrapAxis wrap_axis(uint32_t mode, uint32_t size_log2, uint32_t lo, uint32_t hi)
{
	const int32_t m = (1 << size_log2) - 1;
	switch (mode)
	{
	case WRAP_REPEAT: return { m, 0, INT32_MIN, INT32_MAX };
	case WRAP_CLAMP: return { -1, 0, 0, m };
	case WRAP_REGION_CLAMP: return { -1, 0, int32_t(lo), int32_t(hi) };
	default: return { m & int32_t(lo), int32_t(hi), INT32_MIN, INT32_MAX };
	}
}

__device__ __forceinline__ int32_t wrap_apply(int32_t v, const WrapAxis &w)
{
	return min(max((v & w.and_mask) | w.or_mask, w.lo), w.hi);
}

__device__ __forceinline__ int32_t wrap_coord(int32_t v, uint32_t mode, uint32_t size_log2, uint32_t lo, uint32_t hi)
{
	int32_t size = 1 << size_log2;
	switch (mode)
	{
	case WRAP_REPEAT: return v & (size - 1);
	case WRAP_CLAMP: return min(max(v, 0), size - 1);
	case WRAP_REGION_CLAMP: return min(max(v, int32_t(lo)), int32_t(hi));
	default: return int32_t(((uint32_t(v) & uint32_t(size - 1)) & lo) | hi);
	}
}

// Grid y = texture, z = slot (mip level, or sample layer of a super-sampled
// texture); level l reads from MIPTBP's base and stride (upload_texture's
// per-level loop, gs/gs_renderer.cpp:3543-3590).
__global__ void __launch_bounds__(256) texture_decode_kernel(PassParams P)
{
	const uint32_t tex = blockIdx.y, level = blockIdx.z;
	if (tex >= P.num_textures)
		return;
	const pgs_texture_desc t = P.textures[tex];
	if (level >= texture_slots(t))
		return;
	const TexImage im = P.tex_images[tex * TEX_SLOTS + level];
	const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
	if (i >= im.ext_u * im.ext_v)
		return;
	const int32_t x = int32_t(i % im.ext_u), y = int32_t(i / im.ext_u);
	const uint8_t *src = texture_source(P, tex);
	if (t.samples > 1 && level > 0)
	{
		P.texels[im.offset + i] = fetch_texel_sample(P, src, t, x, y, level - 1u);
		return;
	}
	uint32_t tbp = t.tbp0, tbw = t.tbw;
	if (level)
	{
		tbp = t.mip[level - 1] & 0x3fffu;
		tbw = t.mip[level - 1] >> 16;
	}
	P.texels[im.offset + i] = fetch_texel(P, src, t, tbp, tbw, x, y);
}

// log2 of a positive normal float: ln m = 2 atanh(s), s = (m - 1) / (m + 1),
// by the series s + s^3/3 + ... + s^9/9 with m reduced to [sqrt(1/2), sqrt(2)]
// (|s| <= 0.172, truncation error below 2e-8).  Every operation is rounded on
// its own, so the CPU restatement computes the same bits.
__device__ __forceinline__ float lod_log2(float x)
{
	uint32_t b = f2u(x);
	int32_t e = int32_t((b >> 23) & 0xffu) - 127;
	float m = u2f((b & 0x7fffffu) | 0x3f800000u);
	if (m > 1.41421356f)
	{
		m = fmul(m, 0.5f);
		e++;
	}
	float s = __fdiv_rn(fsub(m, 1.0f), fadd(m, 1.0f));
	float s2 = fmul(s, s);
	float poly = fadd(fmul(s2, 1.0f / 9.0f), 1.0f / 7.0f);
	poly = fadd(fmul(s2, poly), 1.0f / 5.0f);
	poly = fadd(fmul(s2, poly), 1.0f / 3.0f);
	poly = fadd(fmul(s2, poly), 1.0f);
	float ln_m = fmul(fmul(2.0f, s), poly);
	return fadd(__int2float_rn(e), fmul(ln_m, 1.44269504f));
}

// One filtered sample of mip level `level` (exact integer filtering; the
// level's coordinates follow sample_texture, ubershader.comp:1133-1151,
// 1214-1227, with region bounds and masks shifted down by the level as in
// texture_clamp, :947-953, and upload_texture, gs/gs_renderer.cpp:3578-3590).
__device__ void sample_level(const PassParams &P, uint32_t tex_index, const pgs_texture_desc &t, uint32_t level,
                             uint32_t slot, bool clamp_s, bool clamp_t, bool linear, float u, float v, bool perspective,
                             uint32_t rgba[4])
{
	const uint32_t twl = t.tw_log2 - level, thl = t.th_log2 - level;
	float uu, vv;
	if (perspective)
	{
		uu = fmul(u, float(1u << twl));
		vv = fmul(v, float(1u << thl));
	}
	else
	{
		float inv = u2f((127u - level) << 23);
		uu = fmul(u, inv);
		vv = fmul(v, inv);
	}
	const uint32_t minu = t.minu >> level, maxu = t.maxu >> level, minv = t.minv >> level, maxv = t.maxv >> level;
	if (clamp_s)
	{
		uint32_t lo = t.wms == WRAP_REGION_CLAMP ? minu : 0u;
		uint32_t hi = t.wms == WRAP_REGION_CLAMP ? maxu : (1u << twl) - 1u;
		uu = fminf(fmaxf(uu, fadd(float(lo), 0.5f)), fadd(float(hi), 0.5f));
	}
	if (clamp_t)
	{
		uint32_t lo = t.wmt == WRAP_REGION_CLAMP ? minv : 0u;
		uint32_t hi = t.wmt == WRAP_REGION_CLAMP ? maxv : (1u << thl) - 1u;
		vv = fminf(fmaxf(vv, fadd(float(lo), 0.5f)), fadd(float(hi), 0.5f));
	}
	int32_t ku = int32_t(floorf(fadd(fmul(uu, 16.0f), 1.0f / 64.0f)));
	int32_t kv = int32_t(floorf(fadd(fmul(vv, 16.0f), 1.0f / 64.0f)));
	const TexImage im = P.tex_images[tex_index * TEX_SLOTS + slot];
	const uint32_t *img = P.texels + im.offset;
	const WrapAxis wu = wrap_axis(t.wms, twl, minu, maxu), wv = wrap_axis(t.wmt, thl, minv, maxv);
	if (!linear)
	{
		int32_t x = wrap_apply(ku >> 4, wu);
		int32_t y = wrap_apply(kv >> 4, wv);
		uint32_t c = __ldg(img + uint32_t(y) * im.ext_u + uint32_t(x));
		#pragma unroll
		for (int k = 0; k < 4; k++)
			rgba[k] = (c >> (8 * k)) & 0xffu;
		return;
	}
	int32_t bu = ku - 8, bv = kv - 8;
	int32_t x0 = bu >> 4, y0 = bv >> 4;
	uint32_t fx = uint32_t(bu) & 15u, fy = uint32_t(bv) & 15u;
	int32_t xs0 = wrap_apply(x0, wu);
	int32_t xs1 = wrap_apply(x0 + 1, wu);
	int32_t ys0 = wrap_apply(y0, wv);
	int32_t ys1 = wrap_apply(y0 + 1, wv);
	uint32_t w00 = (16u - fx) * (16u - fy), w10 = fx * (16u - fy), w01 = (16u - fx) * fy, w11 = fx * fy;
	const uint32_t *row0 = img + uint32_t(ys0) * im.ext_u, *row1 = img + uint32_t(ys1) * im.ext_u;
	uint32_t c00 = __ldg(row0 + xs0);
	uint32_t c10 = __ldg(row0 + xs1);
	uint32_t c01 = __ldg(row1 + xs0);
	uint32_t c11 = __ldg(row1 + xs1);
	// Two channels per 32-bit word (R and B, then G and A), 16 bits each:
	// the weights sum to 256, so a channel's sum stays below 2^16.
	const uint32_t m = 0x00ff00ffu;
	const uint32_t rb = w00 * (c00 & m) + w10 * (c10 & m) + w01 * (c01 & m) + w11 * (c11 & m);
	const uint32_t ga = w00 * ((c00 >> 8) & m) + w10 * ((c10 >> 8) & m) + w01 * ((c01 >> 8) & m) + w11 * ((c11 >> 8) & m);
	// acc / 256 rounded half to even.
	auto round256 = [](uint32_t acc) { return (acc + 127u + ((acc >> 8) & 1u)) >> 8; };
	rgba[0] = round256(rb & 0xffffu);
	rgba[1] = round256(ga & 0xffffu);
	rgba[2] = round256(rb >> 16);
	rgba[3] = round256(ga >> 16);
}

// Level of detail and filter choice (sample_texture, ubershader.comp:1064-1131):
// LOD = ceil(-log2|Q| * 2^(L+4) + K) / 16 or the fixed K >> 4, clamped to
// [0, MXL]; MMIN applies when the LOD is positive; trilinear blends the next
// level by floor(fract * 16) / 16.  Levels beyond the texture's chain read its
// last level.  Returns level | next level << 4 | weight of the next level << 8
// | linear << 16.
__device__ __forceinline__ uint32_t select_lod(uint32_t levels, uint32_t tex_word, uint32_t tex2, float q)
{
	const bool mag_linear = (tex_word & TEX_SAMPLER_MAG_LINEAR_BIT) != 0;
	const bool min_linear = (tex_word & TEX_SAMPLER_MIN_LINEAR_BIT) != 0;
	const uint32_t max_mip = (tex_word >> TEX_MAX_MIP_LEVEL_OFFSET) & 7u;
	const int32_t K = int32_t(tex2 << 17) >> 20; // signed 12-bit field at bit 3
	float lod;
	bool linear;
	if ((tex2 & TEX2_FIXED_LOD_BIT) == 0)
	{
		const uint32_t L = (tex2 >> 1) & 3u;
		float aq = fabsf(q), formula = 0.0f;
		if (aq >= 1.17549435e-38f && aq <= 3.40282347e38f)
			formula = fadd(fmul(-lod_log2(aq), float(1u << (L + 4))), __int2float_rn(K));
		lod = fmul(ceilf(formula), 0.0625f);
		linear = formula > 0.0f ? min_linear : mag_linear;
	}
	else
	{
		lod = __int2float_rn(K >> 4);
		linear = lod > 0.0f ? min_linear : mag_linear;
	}
	lod = fminf(fmaxf(lod, 0.0f), float(max_mip));
	float l1 = floorf(lod), l2 = ceilf(lod);
	uint32_t weight = uint32_t(fmul(fsub(lod, l1), 16.0f));
	if ((tex_word & TEX_SAMPLER_MIPMAP_LINEAR_BIT) == 0)
	{
		weight = 0;
		l1 = float(int32_t(fadd(lod, 0.5f)));
	}
	const uint32_t last = max(levels, 1u) - 1u;
	return min(uint32_t(l1), last) | (min(uint32_t(l2), last) << 4) | (weight << 8) | (uint32_t(linear) << 16);
}

// MIP: the pass samples mip levels (some primitive has TEX1.MXL > 0 with a
// mipmapping MMIN) or super-sampled textures; without it every sample reads
// level 0 of a plain texture through MMAG.
// Super-sampled texture (ubershader.comp:1155-1212).  Sample mapping reads the
// layer of the shading sample, the resolved bit layer 0; otherwise the phase
// LUT picks up to four (layer, texel) taps around the texel below the
// sampling position, weighted in unorm8 (one tap when filtering is nearest or
// the texel is on a clamped region edge).  Taps wrap like the texture.
__device__ void sample_layered(const PassParams &P, uint32_t tex_index, const pgs_texture_desc &t, uint32_t tex_word,
                               float u, float v, bool perspective, uint32_t sample, uint32_t rx, uint32_t ry,
                               uint32_t rgba[4])
{
	const bool clamp_s = (tex_word & TEX_SAMPLER_CLAMP_S_BIT) != 0;
	const bool clamp_t = (tex_word & TEX_SAMPLER_CLAMP_T_BIT) != 0;
	const bool mag_linear = (tex_word & TEX_SAMPLER_MAG_LINEAR_BIT) != 0;
	if (tex_word & (TEX_SAMPLE_MAPPING_BIT | TEX_SAMPLE_RESOLVED_BIT))
	{
		const uint32_t layer = (tex_word & TEX_SAMPLE_MAPPING_BIT) ? min(sample + 1u, t.samples) : 0u;
		sample_level(P, tex_index, t, 0, layer, clamp_s, clamp_t, mag_linear, u, v, perspective, rgba);
		return;
	}
	const float w = float(1u << t.tw_log2), h = float(1u << t.th_log2);
	float uu = perspective ? fmul(u, w) : u;
	float vv = perspective ? fmul(v, h) : v;
	// Region of the reference's TexInfo (CLAMP: the image, REGION_CLAMP: MIN/MAX, else 0).
	const int32_t rx0 = t.wms == WRAP_REGION_CLAMP ? int32_t(t.minu) : 0;
	const int32_t rx1 = t.wms == WRAP_REGION_CLAMP ? int32_t(t.maxu) : (t.wms == WRAP_CLAMP ? int32_t(w) - 1 : 0);
	const int32_t ry0 = t.wmt == WRAP_REGION_CLAMP ? int32_t(t.minv) : 0;
	const int32_t ry1 = t.wmt == WRAP_REGION_CLAMP ? int32_t(t.maxv) : (t.wmt == WRAP_CLAMP ? int32_t(h) - 1 : 0);
	if (clamp_s)
		uu = fminf(fmaxf(uu, fadd(float(rx0), 0.5f)), fadd(float(rx1), 0.5f));
	if (clamp_t)
		vv = fminf(fmaxf(vv, fadd(float(ry0), 0.5f)), fadd(float(ry1), 0.5f));
	const float shift = fsub(0.5f, average_sampling_offset(rx, ry));
	const float su = fsub(fadd(uu, 1.0f / 1024.0f), shift), sv = fsub(fadd(vv, 1.0f / 1024.0f), shift);
	const float fu = floorf(su), fv = floorf(sv);
	const int32_t ix = int32_t(fu), iy = int32_t(fv);
	const float pu = fsub(su, fu), pv = fsub(sv, fv);
	uint32_t entry, weights = 0;
	if (mag_linear)
	{
		const uint32_t lx = min(uint32_t(fmul(pu, 64.0f)), 63u), ly = min(uint32_t(fmul(pv, 64.0f)), 63u);
		entry = __ldg(P.phase_lut + (ly * 64u + lx) * 2u);
		weights = __ldg(P.phase_lut + (ly * 64u + lx) * 2u + 1u);
	}
	else
	{
		const uint32_t lx = min(uint32_t(fmul(pu, 32.0f)), 31u), ly = min(uint32_t(fmul(pv, 32.0f)), 31u);
		entry = __ldg(P.phase_lut + 64u * 64u * 2u + ly * 32u + lx);
	}
	const bool force_nearest =
	    !mag_linear || ((clamp_s || clamp_t) && (ix == rx0 || iy == ry0 || ix == rx1 || iy == ry1));
	auto tap = [&](uint32_t layer, int32_t x, int32_t y) {
		layer = min(layer + 1u, t.samples);
		const TexImage im = P.tex_images[tex_index * TEX_SLOTS + layer];
		const int32_t wx = wrap_coord(x, t.wms, t.tw_log2, t.minu, t.maxu);
		const int32_t wy = wrap_coord(y, t.wmt, t.th_log2, t.minv, t.maxv);
		return __ldg(P.texels + im.offset + uint32_t(wy) * im.ext_u + uint32_t(wx));
	};
	const uint32_t c0 = tap(entry & 15u, ix, iy);
	if (force_nearest)
	{
		#pragma unroll
		for (int k = 0; k < 4; k++)
			rgba[k] = (c0 >> (8 * k)) & 0xffu;
		return;
	}
	uint32_t acc[4];
	const uint32_t w0 = weights & 0xffu;
	#pragma unroll
	for (int k = 0; k < 4; k++)
		acc[k] = w0 * ((c0 >> (8 * k)) & 0xffu);
	for (uint32_t i = 1; i < 4; i++)
	{
		const uint32_t wi = (weights >> (8 * i)) & 0xffu;
		if (!wi)
			continue;
		const int32_t ox = int32_t(entry << (14 - 4 * i)) >> 30, oy = int32_t(entry << (12 - 4 * i)) >> 30;
		const uint32_t c = tap((entry >> (4 * i)) & 15u, ix + ox, iy + oy);
		#pragma unroll
		for (int k = 0; k < 4; k++)
			acc[k] += wi * ((c >> (8 * k)) & 0xffu);
	}
	// round(acc / 255); a tie would need acc = 255 (2q + 1) / 2.
	#pragma unroll
	for (int k = 0; k < 4; k++)
	{
		const uint32_t q = acc[k] / 255u, r = acc[k] % 255u;
		rgba[k] = q + (2u * r > 255u ? 1u : 0u);
	}
}

template <bool MIP>
__device__ void sample_texture(const PassParams &P, uint32_t tex_word, uint32_t tex2, float u, float v, float q,
                               bool perspective, uint32_t sample, uint32_t rx, uint32_t ry, float out[4])
{
	const uint32_t tex_index = min(tex_word & TEX_TEXTURE_INDEX_MASK, P.num_textures - 1u);
	pgs_texture_desc t = P.textures[tex_index];
	// Descriptors keep only the region modes; plain REPEAT and CLAMP come from
	// the primitive's sampler bits, as the reference's shader takes them
	// (drawing_kick_update_texture, gs/gs_interface.cpp:1514-1528).
	effective_wrap(t, tex_word);
	if (MIP && (tex_word & TEX_PER_SAMPLE_BIT) && t.samples > 1)
	{
		uint32_t rgba[4];
		sample_layered(P, tex_index, t, tex_word, u, v, perspective, sample, rx, ry, rgba);
		#pragma unroll
		for (int k = 0; k < 4; k++)
			out[k] = float(rgba[k]);
		return;
	}
	const bool clamp_s = (tex_word & TEX_SAMPLER_CLAMP_S_BIT) != 0;
	const bool clamp_t = (tex_word & TEX_SAMPLER_CLAMP_T_BIT) != 0;
	if (!MIP)
	{
		// Level 0 through MMAG: the level blend below is the identity.
		uint32_t c[4];
		sample_level(P, tex_index, t, 0, 0, clamp_s, clamp_t, (tex_word & TEX_SAMPLER_MAG_LINEAR_BIT) != 0, u, v,
		             perspective, c);
		#pragma unroll
		for (int k = 0; k < 4; k++)
			out[k] = float(c[k]);
		return;
	}
	uint32_t sel = (tex_word & TEX_SAMPLER_MAG_LINEAR_BIT) ? (1u << 16) : 0u;
	if (MIP && ((tex_word >> TEX_MAX_MIP_LEVEL_OFFSET) & 7u))
		sel = select_lod(t.levels, tex_word, tex2, q);
	// One pass per sampled level: weight 16 - w on the first, w on the second,
	// then roundEven(sum / 16) (exact for a single level).
	const uint32_t weight = (sel >> 8) & 0xffu;
	uint32_t acc[4] = { 0, 0, 0, 0 };
	for (uint32_t pass = 0; pass < (weight ? 2u : 1u); pass++)
	{
		uint32_t c[4];
		const uint32_t lv = pass ? ((sel >> 4) & 15u) : (sel & 15u);
		sample_level(P, tex_index, t, lv, lv, clamp_s, clamp_t, (sel >> 16) != 0, u, v, perspective, c);
		const uint32_t w = pass ? weight : 16u - weight;
		#pragma unroll
		for (int k = 0; k < 4; k++)
			acc[k] += w * c[k];
	}
	#pragma unroll
	for (int k = 0; k < 4; k++)
	{
		uint32_t r = acc[k] >> 4, f = acc[k] & 15u;
		if (f > 8u || (f == 8u && (r & 1u)))
			r++;
		out[k] = float(r);
	}
}

__device__ __forceinline__ float interp(float c0, float d1, float d2, float i, float j)
{
	// c0 + d1 * i + d2 * j, left to right, one rounding per operation.
	return fadd(fadd(c0, fmul(d1, i)), fmul(d2, j));
}

template <bool MIP>
__device__ void combined_color(const ShadeCtx &C, uint32_t pi, const Request &r, bool perspective, uint32_t combiner,
                               float cc[4])
{
	const PassParams &P = *C.P;
	const TransformedAttr a = P.tattr[pi];
	float col[4];
	#pragma unroll
	for (int k = 0; k < 4; k++)
	{
		float t = interp(a.rgba0[k], a.rgba1[k], a.rgba2[k], r.i, r.j);
		col[k] = floorf(fadd(fmul(255.0f, t), 1.0f / 256.0f));
	}
	bool fog = (combiner & COMBINER_FOG_BIT) != 0, tcc = (combiner & COMBINER_TCC_BIT) != 0;
	bool tme = (combiner & COMBINER_TME_BIT) != 0;
	uint32_t mode = combiner & COMBINER_MODE_MASK;
	if (tme)
	{
		float s = interp(a.stqf0[0], a.stqf1[0], a.stqf2[0], r.i, r.j);
		float t = interp(a.stqf0[1], a.stqf1[1], a.stqf2[1], r.i, r.j);
		float q = interp(a.stqf0[2], a.stqf1[2], a.stqf2[2], r.i, r.j);
		if (perspective && q != 1.0f)
		{
			s = __fdiv_rn(s, q);
			t = __fdiv_rn(t, q);
		}
		s = fminf(fmaxf(s, -2047.0f), 2047.0f);
		t = fminf(fmaxf(t, -2047.0f), 2047.0f);
		float tx[4];
		sample_texture<MIP>(P, P.prims[pi].tex, P.prims[pi].tex2, s, t, q, perspective, C.sample,
		                    C.ss ? C.I->rate_x_log2 : 0u, C.ss ? C.I->rate_y_log2 : 0u, tx);
		if (mode == COMBINER_DECAL)
		{
			cc[0] = tx[0]; cc[1] = tx[1]; cc[2] = tx[2]; cc[3] = tcc ? tx[3] : col[3];
		}
		else
		{
			#pragma unroll
			for (int k = 0; k < 4; k++)
				cc[k] = fminf(fmaxf(floorf(fmul(fmul(col[k], tx[k]), 1.0f / 128.0f)), 0.0f), 255.0f);
			if (mode == COMBINER_MODULATE)
			{
				if (!tcc) cc[3] = col[3];
			}
			else
			{
				cc[0] = fadd(cc[0], col[3]); cc[1] = fadd(cc[1], col[3]); cc[2] = fadd(cc[2], col[3]);
				if (mode == COMBINER_HIGHLIGHT)
					cc[3] = tcc ? fadd(tx[3], col[3]) : col[3];
				else
					cc[3] = tcc ? tx[3] : col[3];
				#pragma unroll
				for (int k = 0; k < 4; k++)
					cc[k] = fminf(fmaxf(cc[k], 0.0f), 255.0f);
			}
		}
	}
	else
	{
		cc[0] = col[0]; cc[1] = col[1]; cc[2] = col[2]; cc[3] = col[3];
	}
	if (fog)
	{
		float f = rintf(interp(a.stqf0[3], a.stqf1[3], a.stqf2[3], r.i, r.j));
		uint32_t fc = P.prims[pi].fogcol;
		#pragma unroll
		for (int k = 0; k < 3; k++)
		{
			float fcol = fmul(unorm8_lut(P.unorm_lut, fc, k), 255.0f);
			float d = fmul(fmul(fsub(cc[k], fcol), f), 1.0f / 256.0f);
			cc[k] = floorf(fadd(fadd(fcol, d), 0.5f));
		}
	}
}

struct SampleState
{
	uint32_t color, depth;
	bool color_dirty, depth_dirty;
	int32_t hx, hy;
	Request pending;
	uint32_t pending_prim;
};

template <bool MIP>
__device__ void shade_resolve(const ShadeCtx &C, SampleState &S)
{
	const PassParams &P = *C.P;
	const Request &r = S.pending;
	uint32_t pi = S.pending_prim;
	const uint32_t pst = P.prims[pi].state;
	const pgs_state_vector sv = P.states[min(pst & STATE_INDEX_MASK, P.num_states - 1u)];
	if (C.zs && r.z_test)
	{
		bool pass = ((pst >> STATE_BIT_Z_TEST_GREATER) & 1) ? r.z > S.depth : r.z >= S.depth;
		if (!pass)
			return;
	}
	const bool multisample = (pst >> STATE_BIT_MULTISAMPLE) & 1;
	float cc[4];
	combined_color<MIP>(C, pi, r, (pst >> STATE_BIT_PERSPECTIVE) & 1, sv.combiner, cc);
	float fbc[4];
	#pragma unroll
	for (int k = 0; k < 4; k++)
		fbc[k] = float((S.color >> (8 * k)) & 0xffu); // == round(unorm8(c) * 255) for every byte

	bool write_fb = true, write_zb = true, write_alpha = true;
	const pgs_primitive_attribute &pa = P.prims[pi];
	uint32_t bm = sv.blend_mode;
	bool abe = (bm & BLEND_MODE_ABE_BIT) != 0;
	bool fb24 = psm_is_24bit(C.fb_psm), fb32 = psm_is_32bit(C.fb_psm), fb16 = psm_is_16bit(C.fb_psm);
	uint32_t alpha_word = pa.alpha;

	if (P.has_aa1)
	{
		bool use_cov = (cc[3] == 128.0f || !abe) && multisample;
		if (use_cov)
			cc[3] = float(r.coverage);
		if (multisample)
			abe = true;
	}

	if (bm & BLEND_MODE_ATE_BIT)
	{
		float aref = float(alpha_word & 0xffu);
		float al = cc[3];
		bool pass;
		switch ((bm >> BLEND_MODE_ATE_MODE_OFFSET) & 7u)
		{
		case ATST_NEVER: pass = false; break;
		case ATST_LESS: pass = al < aref; break;
		case ATST_LEQUAL: pass = al <= aref; break;
		case ATST_EQUAL: pass = al == aref; break;
		case ATST_GEQUAL: pass = al >= aref; break;
		case ATST_GREATER: pass = al > aref; break;
		case ATST_NOTEQUAL: pass = al != aref; break;
		default: pass = true; break;
		}
		if (!pass)
		{
			switch ((bm >> BLEND_MODE_AFAIL_MODE_OFFSET) & 3u)
			{
			case AFAIL_KEEP: return;
			case AFAIL_FB_ONLY: write_zb = false; break;
			case AFAIL_ZB_ONLY: write_fb = false; write_alpha = false; break;
			default: if (fb32) write_alpha = false; write_zb = false; break;
			}
		}
	}

	if (!fb24 && (bm & BLEND_MODE_DATE_BIT))
	{
		uint32_t bit = fbc[3] >= 128.0f ? 1u : 0u;
		if (((bm & BLEND_MODE_DATM_BIT) ? 1u : 0u) != bit)
			return;
	}

	if ((bm & BLEND_MODE_PABE_BIT) && cc[3] < 128.0f)
		abe = false;

	float bl[4] = { cc[0], cc[1], cc[2], cc[3] };
	if (abe)
	{
		uint32_t am = (bm >> BLEND_MODE_A_MODE_OFFSET) & 3u, bmo = (bm >> BLEND_MODE_B_MODE_OFFSET) & 3u;
		uint32_t cm = (bm >> BLEND_MODE_C_MODE_OFFSET) & 3u, dm = (bm >> BLEND_MODE_D_MODE_OFFSET) & 3u;
		float Cf = 0.0f;
		if (cm == BLEND_ALPHA_SOURCE) Cf = cc[3];
		else if (cm == BLEND_ALPHA_DEST) Cf = fb24 ? 128.0f : fbc[3];
		else if (cm == BLEND_ALPHA_FIX) Cf = float((alpha_word >> ALPHA_AFIX_OFFSET) & 0xffu);
		#pragma unroll
		for (int k = 0; k < 3; k++)
		{
			float A = am == 0 ? cc[k] : (am == 1 ? fbc[k] : 0.0f);
			float B = bmo == 0 ? cc[k] : (bmo == 1 ? fbc[k] : 0.0f);
			float D = dm == 0 ? cc[k] : (dm == 1 ? fbc[k] : 0.0f);
			bl[k] = fadd(floorf(fmul(fmul(fsub(A, B), Cf), 1.0f / 128.0f)), D);
		}
	}

	if (bm & BLEND_MODE_DTHE_BIT)
	{
		int px = (S.hx >> C.dim) & 3, py = (S.hy >> C.dim) & 3;
		int bit = ((py * 4 + px) * 4) & 31;
		uint32_t dimx = py < 2 ? sv.dimx_lo : sv.dimx_hi;
		int32_t dv = int32_t(((dimx >> bit) & 7u) << 29) >> 29;
		float fdv = float(dv);
		bl[0] = fadd(bl[0], fdv); bl[1] = fadd(bl[1], fdv); bl[2] = fadd(bl[2], fdv);
	}

	if (fb24) write_alpha = false;
	if (!write_alpha) bl[3] = fbc[3];
	if (!write_fb) { bl[0] = fbc[0]; bl[1] = fbc[1]; bl[2] = fbc[2]; }

	float o[4];
	bool colclamp = (bm & BLEND_MODE_COLCLAMP_BIT) != 0;
	#pragma unroll
	for (int k = 0; k < 4; k++)
	{
		if (!colclamp)
		{
			float x = fmul(bl[k], 1.0f / 256.0f);
			o[k] = fmul(fsub(x, floorf(x)), 256.0f / 255.0f);
		}
		else
			o[k] = fmul(bl[k], 1.0f / 255.0f);
	}
	uint32_t packed = pack_unorm(o[0], o[1], o[2], o[3]);
	if ((bm & BLEND_MODE_FB_ALPHA_BIT) && write_alpha)
		packed |= 0x80000000u;

	uint32_t mask = pa.fbmsk;
	if (mask != 0xffffffffu && (write_fb || write_alpha))
	{
		S.color = mask ? ((packed & ~mask) | (S.color & mask)) : packed;
		if (fb16)
			S.color &= 0x80f8f8f8u;
		S.color_dirty = true;
	}
	if (C.zs && write_zb && r.z_write)
	{
		S.depth = r.z;
		S.depth_dirty = true;
	}
}

// Coverage of one sample for primitives without AA1 (evaluate_coverage with
// multisample == false): 0x80 when the sample is inside, else 0.  The
// barycentrics are computed separately, only once some lane is covered.
__device__ __forceinline__ int coverage_plain(const PrimSetup &s, int32_t cx, int32_t cy, int dim)
{
	int32_t sx = cx >> dim, sy = cy >> dim;
	if (!(sx >= s.bb[0] && sy >= s.bb[1] && s.bb[2] >= sx && s.bb[3] >= sy))
		return 0;
	int32_t axw = s.a[0];
	int32_t A[3] = { axw >> 6, s.a[1], s.a[2] };
	int32_t px = cx << (3 - dim), py = cy << (3 - dim);
	int32_t ea = idot3(A, px, py), eb = idot3(s.b, px, py), ec = idot3(s.c, px, py);
	if ((axw & 1) && ea < 0)
	{
		eb += ea + int32_t((uint32_t(axw) >> 2) & 3u) - 1;
		ec += ea + int32_t((uint32_t(axw) >> 4) & 3u) - 1;
		ea = 0;
	}
	return (ea >= 0 && eb >= 0 && ec >= 0) ? 0x80 : 0;
}

__device__ __forceinline__ int evaluate_coverage(const PrimSetup &s, int32_t cx, int32_t cy, float &i, float &j, bool ms,
                                                 bool line, int dim)
{
	int32_t sx = cx >> dim, sy = cy >> dim;
	if (!(sx >= s.bb[0] && sy >= s.bb[1] && s.bb[2] >= sx && s.bb[3] >= sy))
		return 0;
	int32_t axw = s.a[0];
	bool par = (axw & 1) != 0;
	int32_t off_b = int32_t((uint32_t(axw) >> 2) & 3u) - 1;
	int32_t off_c = int32_t((uint32_t(axw) >> 4) & 3u) - 1;
	int32_t A[3] = { axw >> 6, s.a[1], s.a[2] };
	int32_t px = cx << (3 - dim), py = cy << (3 - dim);
	int32_t ea = idot3(A, px, py), eb = idot3(s.b, px, py), ec = idot3(s.c, px, py);
	i = fadd(fmul(__int2float_rn(eb), s.inv_area), s.error_i);
	j = fadd(fmul(__int2float_rn(ec), s.inv_area), s.error_j);
	bool ba = ea >= 0, bb = eb >= 0, bc = ec >= 0;
	if (par && ea < 0)
	{
		eb += ea + off_b;
		ec += ea + off_c;
		ea = 0;
	}
	bool center = ea >= 0 && eb >= 0 && ec >= 0;
	if (ms && line)
		return center ? int(fmaxf(0.0f, fsub(128.0f, fmul(256.0f, fabsf(fsub(0.5f, j)))))) : 0;
	if (center)
		return 0x80;
	if (ms && !par && (int(ba) + int(bb) + int(bc) == 2))
	{
		float neg;
		int32_t md;
		if (!ba)
		{
			md = max(abs(s.b[0] + s.c[0]), abs(s.b[1] + s.c[1]));
			neg = fsub(fadd(i, j), 1.0f);
		}
		else if (!bb)
		{
			md = max(abs(s.b[0]), abs(s.b[1]));
			neg = -i;
		}
		else
		{
			md = max(abs(s.c[0]), abs(s.c[1]));
			neg = -j;
		}
		float scaled = fmul(float(md), s.inv_area);
		float fc = fsub(8.0f, __fdiv_rn(neg, scaled));
		return int(fminf(fmaxf(fmul(16.0f, fc), 0.0f), 127.0f));
	}
	return 0;
}

// Must be called by all lanes of a warp; returns with warp_any == false (and no
// further work) when no lane of the warp is covered.  AA compiles the AA1
// coverage path in (ubershader variant VARIANT_FLAG_HAS_AA1_BIT).
template <bool AA, bool TEX_ARRAY>
__device__ __forceinline__ Request shade_early(const ShadeCtx &C, const PrimSetup &s, uint32_t pi, uint32_t st,
                                               const SampleState &S, bool &opaque, bool &warp_any)
{
	const PassParams &P = *C.P;
	Request r;
	opaque = (st >> STATE_BIT_OPAQUE) & 1;
	r.z_test = C.zs && ((st >> STATE_BIT_Z_TEST) & 1);
	r.z_write = C.zs && ((st >> STATE_BIT_Z_WRITE) & 1);
	const bool multisample = AA && ((st >> STATE_BIT_MULTISAMPLE) & 1);
	int32_t rx = S.hx, ry = S.hy;
	if (C.ss && (st & (1u << STATE_BIT_SNAP_RASTER)))
	{
		// Sample-mapped textures keep the full-rate row grid when rows are
		// snapped for field rendering (ubershader.comp:816-821).
		rx &= C.snap_mask_x;
		ry &= (TEX_ARRAY && (P.prims[pi].tex & TEX_SAMPLE_MAPPING_BIT)) ? C.snap_mask_x : C.snap_mask_y;
	}
	float i = 0.0f, j = 0.0f;
	if (AA)
		r.coverage = evaluate_coverage(s, rx, ry, i, j, multisample, (st >> STATE_BIT_LINE) & 1, C.dim);
	else
		r.coverage = coverage_plain(s, rx, ry, C.dim);
	if (P.has_scanmsk)
	{
		int32_t sy = S.hy;
		if (st & (1u << STATE_BIT_SPRITE))
			sy >>= C.dim;
		if ((sy & 1) == 0) { if ((st >> STATE_BIT_SCANMSK_EVEN) & 1) r.coverage = 0; }
		else if ((st >> STATE_BIT_SCANMSK_ODD) & 1) r.coverage = 0;
	}
	warp_any = __any_sync(0xffffffffu, r.coverage > 0);
	if (!warp_any)
		return r;
	if (!AA)
	{
		// Barycentrics at the raster coordinate (evaluate_coverage_single).
		int32_t qx = rx << (3 - C.dim), qy = ry << (3 - C.dim);
		i = fadd(fmul(__int2float_rn(idot3(s.b, qx, qy)), s.inv_area), s.error_i);
		j = fadd(fmul(__int2float_rn(idot3(s.c, qx, qy)), s.inv_area), s.error_j);
	}
	if (C.zs && multisample && r.coverage < 0x80)
		r.z_write = false;
	uint32_t z = s.z[0];
	float zf = rintf(fadd(fmul(u2f(s.z[1]), i), fmul(u2f(s.z[2]), j)));
	zf = fminf(fmaxf(zf, 0.0f), 4294967040.0f);
	uint32_t dz = __float2uint_rz(zf);
	dz = min(dz, 0xffffffffu - z);
	z += dz;
	if (C.zs && psm_is_16bit(C.zb_psm)) z = min(z, 0xffffu);
	else if (C.zs && psm_is_24bit(C.zb_psm)) z = min(z, 0xffffffu);
	if (C.ss && r.coverage != 0)
	{
		uint32_t snap = st & ((1u << STATE_BIT_SNAP_RASTER) | (1u << STATE_BIT_SNAP_ATTRIBUTE));
		if (snap == (1u << STATE_BIT_SNAP_ATTRIBUTE))
		{
			int32_t qx = (S.hx & C.snap_mask_x) << (3 - C.dim), qy = (S.hy & C.snap_mask_y) << (3 - C.dim);
			i = fadd(fmul(__int2float_rn(idot3(s.b, qx, qy)), s.inv_area), s.error_i);
			j = fadd(fmul(__int2float_rn(idot3(s.c, qx, qy)), s.inv_area), s.error_j);
		}
		else if (TEX_ARRAY && snap == (1u << STATE_BIT_SNAP_RASTER))
		{
			// Per-sample textured sprite: coverage snapped, attributes
			// interpolated per sample (ubershader.comp:888-895).
			int32_t qx = S.hx << (3 - C.dim), qy = S.hy << (3 - C.dim);
			i = fadd(fmul(__int2float_rn(idot3(s.b, qx, qy)), s.inv_area), s.error_i);
			j = fadd(fmul(__int2float_rn(idot3(s.c, qx, qy)), s.inv_area), s.error_j);
		}
	}
	r.z = z;
	r.i = i;
	r.j = j;
	return r;
}

// Sample position within its pixel for sample s (32-wide subgroup layout of
// ubershader.comp get_tile_info, :253-340).  Ordered grids interleave x/y
// lane bits; a 2:1 grid is a checkerboard; a 4:1 grid puts one sample per
// high-res row at x offsets 0, 2, 3, 1 (the 0x78 pattern, :333-338).
__device__ __forceinline__ void sample_offset(uint32_t s, uint32_t xl, uint32_t yl, int32_t &ox, int32_t &oy)
{
	uint32_t b0 = s & 1u, b1 = (s >> 1) & 1u, b2 = (s >> 2) & 1u, b3 = (s >> 3) & 1u;
	if (xl == yl)
	{
		ox = int32_t(b1 | (b3 << 1));
		oy = int32_t(b0 | (b2 << 1));
	}
	else if (yl == xl + 2)
	{
		oy = int32_t(s & ((1u << yl) - 1u));
		ox = int32_t(((s >> yl) << 2) + ((0x78u >> ((oy & 3) * 2)) & 3u));
	}
	else
	{
		int32_t ly = int32_t(b0 | (xl >= 1 ? (b2 << 1) : 0u));
		int32_t lx = int32_t(xl >= 1 ? b1 : 0u);
		ox = (lx << 1) + (ly & 1);
		oy = ly;
	}
}

// Processes one primitive for the calling warp: coverage, early depth,
// deferred-shading bookkeeping (ubershader.comp:1694-1812).  Warp-uniform.
// The 8x8 bins already hold only primitives that intersect the sub-tile
// (primitive_intersects_tile); a second test against each warp's smaller
// rectangle costs more than the coverage test it would skip, so coverage
// alone decides.
template <bool SS, bool AA, bool MIP>
__device__ __forceinline__ void process_primitive_with(const ShadeCtx &C, uint32_t pi, const PrimSetup &s, uint32_t st,
                                                       SampleState &S, uint32_t &covered)
{
	bool opaque, any_cov;
	Request q = shade_early<AA, MIP>(C, s, pi, st, S, opaque, any_cov);
	if (!any_cov)
		return;
	// A primitive that is not opaque (warp-uniform: a state bit) is shaded
	// right away rather than left pending.  The result is the same as shading
	// it at the next flush: leaving it pending only saves work when a later
	// opaque primitive covers the sample, which blended primitives seldom
	// meet, and shading now keeps every lane of the call on the same
	// primitive.  What was pending is shaded first wherever this primitive
	// covers a sample that has a pending one.  The super-sampled variants take
	// this path on its own; the single-sampled one keeps the shared path below
	// (measured: the separate path speeds the first up and slows the second).
	if (SS && !opaque)
	{
		if (q.coverage > 0)
		{
			covered++;
			if (q.z_test && !S.pending.z_write)
			{
				const bool zp = ((st >> STATE_BIT_Z_TEST_GREATER) & 1) ? q.z > S.depth : q.z >= S.depth;
				if (!zp)
				{
					q.coverage = 0;
					q.z_write = false;
				}
				q.z_test = false;
			}
		}
		if (__any_sync(0xffffffffu, q.coverage > 0 && S.pending.coverage > 0))
		{
			if (S.pending.coverage > 0)
				shade_resolve<MIP>(C, S);
			S.pending.coverage = 0;
			S.pending.z_write = false;
		}
		if (__any_sync(0xffffffffu, q.coverage > 0))
		{
			if (q.coverage > 0)
			{
				S.pending = q;
				S.pending_prim = pi;
				shade_resolve<MIP>(C, S);
				S.pending.coverage = 0;
				S.pending.z_write = false;
			}
		}
		return;
	}
	if (q.coverage > 0)
	{
		covered++;
		if (q.z_test && !S.pending.z_write)
		{
			q.z_test = false;
			bool zp = ((st >> STATE_BIT_Z_TEST_GREATER) & 1) ? q.z > S.depth : q.z >= S.depth;
			if (zp)
			{
				if (q.z_write && opaque)
				{
					q.z_write = false;
					S.depth = q.z;
					S.depth_dirty = true;
				}
			}
			else
			{
				q.coverage = 0;
				q.z_write = false;
			}
		}
		else if (q.z_write && !q.z_test && opaque)
		{
			q.z_write = false;
			S.pending.z_write = false;
			S.depth = q.z;
			S.depth_dirty = true;
		}
		if ((q.z_test || !q.z_write) && S.pending.z_write)
			opaque = false;
	}
	bool need_flush = false;
	if (q.coverage > 0)
	{
		need_flush = !opaque && S.pending.coverage > 0;
		if (!need_flush)
		{
			S.pending = q;
			S.pending_prim = pi;
			q.coverage = 0;
		}
	}
	if (__any_sync(0xffffffffu, need_flush))
	{
		if (S.pending.coverage > 0)
			shade_resolve<MIP>(C, S);
		S.pending.coverage = 0;
		S.pending.z_write = false;
		if (q.coverage > 0)
		{
			S.pending = q;
			S.pending_prim = pi;
		}
	}
	// The shared path shades a primitive that is not opaque at once too.
	if (!((st >> STATE_BIT_OPAQUE) & 1u) &&
	    __any_sync(0xffffffffu, S.pending.coverage > 0 && S.pending_prim == pi))
	{
		if (S.pending.coverage > 0 && S.pending_prim == pi)
		{
			shade_resolve<MIP>(C, S);
			S.pending.coverage = 0;
			S.pending.z_write = false;
		}
	}
}

template <bool SS, bool AA, bool MIP>
__device__ __forceinline__ void process_primitive(const ShadeCtx &C, uint32_t pi, SampleState &S, uint32_t &covered)
{
	const PassParams &P = *C.P;
	const PrimSetup s = P.setup[pi];
	process_primitive_with<SS, AA, MIP>(C, pi, s, P.prims[pi].state, S, covered);
}

// ---------------------------------------------------------------------------
// Primitive culling per warp.  A warp's samples have raster positions (after
// any snapping of coverage) inside a rectangle; a primitive whose box misses
// it, or one of whose edges is negative at every point of it, covers none of
// the warp's samples and would be a no-op for that warp.  The edge test
// follows the coverage test's 32-bit wrapping arithmetic: the value at the
// rectangle's best corner is exact modulo 2^32, every other sample's value
// is that minus at most d, and a primitive is only dropped when no sample's
// value can wrap back to non-negative.

// Whether edge e can be non-negative somewhere in r (raster units, shift sh
// to the coverage test's sub-pixel units).
__device__ __forceinline__ bool edge_may_pass(const int32_t e[3], int4 r, int sh)
{
	const int32_t x = e[0] >= 0 ? r.z : r.x, y = e[1] >= 0 ? r.w : r.y;
	const int32_t v = idot3(e, x << sh, y << sh);
	if (v >= 0)
		return true;
	const int64_t d = llabs(int64_t(e[0])) * (int64_t(r.z - r.x) << sh) + llabs(int64_t(e[1])) * (int64_t(r.w - r.y) << sh);
	return int64_t(v) - d < -2147483648LL;
}

// Conservative: false only when the primitive covers no sample whose raster
// position lies in r = (x0, y0, x1, y1).  Parallelograms (sprites, lines,
// fused rectangles) shift edges past the diagonal and AA1 multisampled
// edges cover outside the triangle, so those keep to the box test.
template <bool AA>
__device__ __forceinline__ bool may_cover(const PrimSetup &s, uint32_t st, int4 r, int dim)
{
	if ((r.z >> dim) < s.bb[0] || (r.x >> dim) > s.bb[2] || (r.w >> dim) < s.bb[1] || (r.y >> dim) > s.bb[3])
		return false;
	if (((st >> STATE_BIT_PARALLELOGRAM) & 1u) || (AA && ((st >> STATE_BIT_MULTISAMPLE) & 1u)))
		return true;
	const int sh = 3 - dim;
	const int32_t A[3] = { s.a[0] >> 6, s.a[1], s.a[2] };
	return edge_may_pass(A, r, sh) && edge_may_pass(s.b, r, sh) && edge_may_pass(s.c, r, sh);
}

// The sub-tile's primitive list, expanded by the whole CTA into primitive
// indices in ascending order in shared memory (CAP at a time), then walked by
// each warp on its own, 32 primitives at a time: every lane tests one
// primitive against the warp's rectangle and the warp shades, in order, the
// primitives that can touch it.  The primitives a warp skips are the ones
// whose coverage test would fail on every lane, so each warp sees the same
// sequence of covering primitives as walking the whole list.  Expansion:
// each warp counts the primitives under its summary words, warp 0 turns the
// counts into offsets, and each warp writes its indices at those offsets.
template <int NS, bool SS, bool AA, bool MIP>
__device__ __forceinline__ void walk_culled(const ShadeCtx &C, const DevInstance &I, const uint32_t *summary,
                                            const uint32_t *mask, uint32_t t, SampleState &S, uint32_t &covered)
{
	constexpr uint32_t T = 64u * NS, WARPS = T / 32u, CAP = 2048u;
	// One summary word per 32 mask words of 32 primitives.
	constexpr uint32_t MAX_SW = (PGS_MAX_PRIMITIVES_PER_FLUSH + 1023u) / 1024u;
	__shared__ uint32_t s_ids[CAP];
	__shared__ uint32_t s_off[MAX_SW + 1];
	__shared__ int4 s_rect[WARPS];
	const PassParams &P = *C.P;
	const uint32_t lane = t & 31u, warp = t >> 5;
	const unsigned full = 0xffffffffu;
	const uint32_t SW = I.summary_words;
	{
		const int32_t x0 = S.hx & C.snap_mask_x, y0 = S.hy & C.snap_mask_x & C.snap_mask_y;
		const int4 r = make_int4(__reduce_min_sync(full, x0), __reduce_min_sync(full, y0),
		                         __reduce_max_sync(full, S.hx), __reduce_max_sync(full, S.hy));
		if (lane == 0)
			s_rect[warp] = r;
	}
	for (uint32_t sw = warp; sw < SW; sw += WARPS)
	{
		const uint32_t words = __ldg(summary + sw);
		const uint32_t mw = ((words >> lane) & 1u) ? __ldg(mask + sw * 32u + lane) : 0u;
		const uint32_t c = __reduce_add_sync(full, uint32_t(__popc(mw)));
		if (lane == 0)
			s_off[sw] = c;
	}
	__syncthreads();
	if (warp == 0)
	{
		uint32_t carry = 0;
		for (uint32_t base = 0; base < SW; base += 32u)
		{
			const uint32_t i = base + lane;
			const uint32_t v = i < SW ? s_off[i] : 0u;
			uint32_t x = v;
			#pragma unroll
			for (int o = 1; o < 32; o <<= 1)
			{
				const uint32_t y = __shfl_up_sync(full, x, o);
				if (lane >= uint32_t(o))
					x += y;
			}
			if (i < SW)
				s_off[i] = carry + x - v;
			carry += __shfl_sync(full, x, 31);
		}
		if (lane == 0)
			s_off[SW] = carry;
	}
	__syncthreads();
	const uint32_t total = s_off[SW];
	for (uint32_t round = 0; round < total; round += CAP)
	{
		for (uint32_t sw = warp; sw < SW; sw += WARPS)
		{
			const uint32_t off = s_off[sw], end = s_off[sw + 1];
			if (end <= round || off >= round + CAP)
				continue;
			const uint32_t words = __ldg(summary + sw);
			const uint32_t mw = ((words >> lane) & 1u) ? __ldg(mask + sw * 32u + lane) : 0u;
			const uint32_t pc = uint32_t(__popc(mw));
			uint32_t x = pc;
			#pragma unroll
			for (int o = 1; o < 32; o <<= 1)
			{
				const uint32_t y = __shfl_up_sync(full, x, o);
				if (lane >= uint32_t(o))
					x += y;
			}
			uint32_t pos = off + x - pc;
			const uint32_t prim_base = I.prim_lo + (sw * 32u + lane) * 32u;
			for (uint32_t m = mw; m; m &= m - 1u, pos++)
				if (pos >= round && pos < round + CAP)
					s_ids[pos - round] = prim_base + uint32_t(__ffs(m) - 1);
		}
		__syncthreads();
		const uint32_t n = min(total - round, CAP);
		for (uint32_t kb = 0; kb < n; kb += 32u)
		{
			const uint32_t k = kb + lane;
			uint32_t pi = 0;
			bool hit = false;
			if (k < n)
			{
				pi = s_ids[k];
				hit = may_cover<AA>(P.setup[pi], P.prims[pi].state, s_rect[warp], C.dim);
			}
			uint32_t bits = __ballot_sync(full, hit);
			while (bits)
			{
				const int b = __ffs(bits) - 1;
				bits &= bits - 1u;
				process_primitive<SS, AA, MIP>(C, __shfl_sync(full, pi, b), S, covered);
			}
		}
		if (round + CAP < total)
			__syncthreads();
	}
}

// One CTA per 8x8-pixel sub-tile, NS samples per pixel, one thread per sample.
// Each warp walks the sub-tile's primitive bitmask on its own (no shared
// memory, no barriers).  SS selects the super-sampled path; sub-tiles whose
// coarse tile selects the other path exit immediately.
// Coarse-tile state of sub-tile `sub`: 0 = empty, 1 = single-sampled,
// 2 = super-sampled (binning.comp:272-311 decision).
__device__ __forceinline__ uint32_t subtile_mode(const PassParams &P, const DevInstance &I, const uint32_t *tile_flags,
                                                 uint32_t sub)
{
	const uint32_t gx = sub % I.sub_w, gy = sub / I.sub_w;
	const uint32_t sh = P.tile_size_log2 - 3u;
	const uint32_t flags = tile_flags[(gy >> sh) * I.tiles_w + (gx >> sh)];
	if (!(flags & TILE_NONEMPTY))
		return 0;
	bool req = I.force_ss || (flags & TILE_REQ_SS);
	if (I.blend_demote && (flags >> TILE_COUNT_SHIFT) >= I.blend_demote && !(flags & TILE_HAS_ZW))
		req = false;
	req = req || ((flags & TILE_REQ_SS_ZW) && (flags & TILE_HAS_ZW));
	return (I.rate_y_log2 != 0 && req) ? 2u : 1u;
}

// One sub-tile's pixel samples; `t` is the thread's index among the 64 * NS
// threads that cover the sub-tile.  CULL: the whole CTA runs the sub-tile and
// walks its primitive list together (walk_culled); otherwise each warp walks
// the sub-tile's primitive bitmask on its own and needs no barrier.
template <int NS, bool SS, bool AA, bool MIP = false, bool CULL = false>
__device__ __forceinline__ void shade_subtile(const PassParams &P, const DevInstance &I, const uint32_t *sub_masks,
                                              const uint32_t *sub_summary, uint32_t sub, uint32_t t)
{
	const uint32_t gx = sub % I.sub_w, gy = sub / I.sub_w;
	const uint32_t *summary = sub_summary + size_t(sub) * I.summary_words;
	const uint32_t *mask = sub_masks + size_t(sub) * I.mask_words;

	ShadeCtx C;
	C.P = &P;
	C.I = &I;
	C.ss = SS;
	C.dim = SS ? int(I.rate_y_log2) : 0;
	C.snap_mask_x = -(1 << I.rate_y_log2);
	C.snap_mask_y = I.snap_mask_y;
	C.zs = I.zb_psm != 0xffffffffu;
	C.fb_psm = I.fb_psm;
	C.zb_psm = I.zb_psm;

	const int32_t sub_x = I.base_x + int32_t(gx * 8u), sub_y = I.base_y + int32_t(gy * 8u);
	const uint32_t lane = t & 31u;
	const uint32_t sample = t % NS;
	C.sample = SS ? sample : 0u;
	const uint32_t pix = t / NS;
	// Pixel order inside the sub-tile: x from bits 0,2,4 and y from bits 1,3,5,
	// so that each warp covers a compact block.
	const int32_t lx = int32_t((pix & 1u) | ((pix >> 1) & 2u) | ((pix >> 2) & 4u));
	const int32_t ly = int32_t(((pix >> 1) & 1u) | ((pix >> 2) & 2u) | ((pix >> 3) & 4u));
	const int32_t px = sub_x + lx, py = sub_y + ly;

	SampleState S;
	int32_t ox = 0, oy = 0;
	if (SS)
		sample_offset(sample, I.rate_x_log2, I.rate_y_log2, ox, oy);
	S.hx = (px << C.dim) + ox;
	S.hy = (py << C.dim) + oy;
	S.color_dirty = false;
	S.depth_dirty = false;
	S.pending.coverage = 0;
	S.pending.z_write = false;
	S.pending_prim = 0;

	const uint32_t fb_index = swizzle_address(uint32_t(px), uint32_t(py), I.fb_base, I.fb_stride, I.fb_psm);
	const uint32_t z_index = C.zs ? swizzle_address(uint32_t(px), uint32_t(py), I.zb_base, I.fb_stride, I.zb_psm) : 0u;
	const uint32_t V32 = VRAM_SIZE / 4, V16 = VRAM_SIZE / 2;
	uint32_t *vram32 = reinterpret_cast<uint32_t *>(P.vram);
	uint16_t *vram16 = reinterpret_cast<uint16_t *>(P.vram);

	// begin_tile
	if (psm_is_16bit(I.fb_psm))
	{
		uint32_t col = vram16[fb_index];
		if (SS && vram16[fb_index + V16] == 0xffffu)
			col = vram16[fb_index + (sample + 2u) * V16];
		S.color = expand16(col);
	}
	else
	{
		S.color = vram32[fb_index];
		if (SS)
		{
			uint32_t ref = vram32[fb_index + V32];
			uint32_t rm = psm_is_24bit(I.fb_psm) ? 0xffffffu : 0xffffffffu;
			if ((ref & rm) == rm)
			{
				uint32_t sc = vram32[fb_index + (sample + 2u) * V32];
				S.color = (psm_is_24bit(I.fb_psm) && ref != 0xffffffffu) ? ((S.color & 0xff000000u) | (sc & 0xffffffu)) : sc;
			}
		}
	}
	if (C.zs)
	{
		const uint8_t *zsrc = P.zcache ? P.zcache : P.vram;
		const uint32_t *z32 = reinterpret_cast<const uint32_t *>(zsrc);
		const uint16_t *z16 = reinterpret_cast<const uint16_t *>(zsrc);
		if (psm_is_16bit(I.zb_psm))
		{
			S.depth = z16[z_index];
			if (SS && z16[z_index + V16] == 0xffffu)
				S.depth = z16[z_index + (sample + 2u) * V16];
		}
		else
		{
			uint32_t rm = psm_is_24bit(I.zb_psm) ? 0xffffffu : 0xffffffffu;
			S.depth = z32[z_index] & rm;
			if (SS && (z32[z_index + V32] & rm) == rm)
				S.depth = z32[z_index + (sample + 2u) * V32] & rm;
		}
	}
	else
		S.depth = 0;

	// Walk the primitive list in ascending order: summary word -> mask words -> bits.
	uint32_t covered = 0;
	if constexpr (CULL)
		walk_culled<NS, SS, AA, MIP>(C, I, summary, mask, t, S, covered);
	else
	for (uint32_t sbase = 0; sbase < I.summary_words; sbase += 32u)
	{
		uint32_t sv = (sbase + lane < I.summary_words) ? __ldg(summary + sbase + lane) : 0u;
		uint32_t nz_lanes = __ballot_sync(0xffffffffu, sv != 0u);
		while (nz_lanes)
		{
			int l = __ffs(nz_lanes) - 1;
			nz_lanes &= nz_lanes - 1u;
			uint32_t words = __shfl_sync(0xffffffffu, sv, l);
			uint32_t word_base = (sbase + uint32_t(l)) * 32u;
			uint32_t mw = ((words >> lane) & 1u) ? __ldg(mask + word_base + lane) : 0u;
			while (words)
			{
				int j = __ffs(words) - 1;
				words &= words - 1u;
				uint32_t m = __shfl_sync(0xffffffffu, mw, j);
				uint32_t prim_base = I.prim_lo + (word_base + uint32_t(j)) * 32u;
				while (m)
				{
					int b = __ffs(m) - 1;
					m &= m - 1u;
					process_primitive<SS, AA, MIP>(C, prim_base + uint32_t(b), S, covered);
				}
			}
		}
	}

	if (S.pending.coverage > 0)
		shade_resolve<MIP>(C, S);

	// Covered-sample counter: one atomic per warp.
	{
		uint32_t c = covered;
		#pragma unroll
		for (int o = 16; o >= 1; o >>= 1)
			c += __shfl_xor_sync(0xffffffffu, c, o);
		if (lane == 0 && c)
			atomicAdd(P.fragment_counter, (unsigned long long)c);
	}

	// end_tile
	const unsigned full = 0xffffffffu;
	uint32_t group_lane0 = (t & 31u) & ~uint32_t(NS - 1);
	bool req_color = false, req_depth = false;
	bool color_dirty = S.color_dirty, depth_dirty = S.depth_dirty;
	uint32_t color = S.color, depth = S.depth;
	uint32_t group_mask = (NS == 32) ? full : (((1u << NS) - 1u) << group_lane0);

	if (SS)
	{
		uint32_t first = __shfl_sync(full, S.color, int(group_lane0));
		req_color = I.preserve_samples ? true : ((__ballot_sync(full, first != S.color) & group_mask) != 0u);
		if (C.zs)
		{
			uint32_t zfirst = __shfl_sync(full, S.depth, int(group_lane0));
			req_depth = (__ballot_sync(full, zfirst != S.depth) & group_mask) != 0u;
		}
		color_dirty = (__ballot_sync(full, S.color_dirty) & group_mask) != 0u;
		// Butterfly sums in the order XOR NS/2 ... 1; every lane takes part.
		const float *lut = P.unorm_lut;
		float v0 = unorm8_lut(lut, S.color, 0), v1 = unorm8_lut(lut, S.color, 1), v2 = unorm8_lut(lut, S.color, 2), v3 = unorm8_lut(lut, S.color, 3);
		#pragma unroll
		for (int o = NS / 2; o >= 1; o >>= 1)
		{
			v0 = fadd(v0, __shfl_xor_sync(full, v0, o));
			v1 = fadd(v1, __shfl_xor_sync(full, v1, o));
			v2 = fadd(v2, __shfl_xor_sync(full, v2, o));
			v3 = fadd(v3, __shfl_xor_sync(full, v3, o));
		}
		float n = float(NS);
		uint32_t resolved = pack_unorm(__fdiv_rn(v0, n), __fdiv_rn(v1, n), __fdiv_rn(v2, n), __fdiv_rn(v3, n));
		uint32_t zmin = S.depth;
		#pragma unroll
		for (int o = NS / 2; o >= 1; o >>= 1)
			zmin = min(zmin, __shfl_xor_sync(full, zmin, o));
		if (C.zs)
			depth_dirty = (__ballot_sync(full, S.depth_dirty) & group_mask) != 0u;

		if (req_color)
		{
			if (color_dirty)
			{
				if (psm_is_16bit(I.fb_psm))
					vram16[fb_index + (sample + 2u) * V16] = uint16_t(rgba32_to_rgba16(S.color));
				else
					vram32[fb_index + (sample + 2u) * V32] = S.color;
			}
			color = I.preserve_samples ? first : resolved;
		}
		if (C.zs && req_depth)
		{
			if (depth_dirty)
			{
				if (psm_is_16bit(I.zb_psm))
					vram16[z_index + (sample + 2u) * V16] = uint16_t(S.depth);
				else
					vram32[z_index + (sample + 2u) * V32] = S.depth;
			}
			depth = zmin;
		}
	}

	bool first_sample = !SS || sample == 0;
	if (color_dirty && first_sample)
	{
		if (psm_is_16bit(I.fb_psm))
		{
			if (P.has_ss_reference)
				vram16[fb_index + V16] = req_color ? 0xffffu : 0u;
			vram16[fb_index] = uint16_t(rgba32_to_rgba16(color));
		}
		else
		{
			if (P.has_ss_reference)
				vram32[fb_index + V32] = req_color ? 0xffffffffu : 0u;
			vram32[fb_index] = color;
		}
	}
	if (C.zs && depth_dirty && first_sample)
	{
		if (psm_is_16bit(I.zb_psm))
		{
			if (P.has_ss_reference)
				vram16[z_index + V16] = req_depth ? 0xffffu : 0u;
			vram16[z_index] = uint16_t(depth);
		}
		else
		{
			if (P.has_ss_reference)
				vram32[z_index + V32] = req_depth ? (psm_is_24bit(I.zb_psm) ? 0xffffffu : 0xffffffffu) : 0u;
			if (psm_is_24bit(I.zb_psm))
			{
				uint8_t *b = P.vram + size_t(z_index) * 4u;
				*reinterpret_cast<uint16_t *>(b) = uint16_t(depth);
				b[2] = uint8_t(depth >> 16);
			}
			else
				vram32[z_index] = depth;
		}
	}
}

template <int NS, bool SS, bool AA, bool MIP>
__global__ void __launch_bounds__(64 * NS, PGS_SHADE_MIN_BLOCKS(NS, AA || MIP)) shade_kernel(PassParams P, DevInstance I, const uint32_t *sub_masks,
                                                        const uint32_t *sub_summary, const uint32_t *tile_flags)
{
	const uint32_t sub = blockIdx.x;
	if (sub >= I.sub_w * I.sub_h)
		return;
	if (subtile_mode(P, I, tile_flags, sub) != (SS ? 2u : 1u))
		return;
	shade_subtile<NS, SS, AA, MIP, true>(P, I, sub_masks, sub_summary, sub, threadIdx.x);
}

// ---------------------------------------------------------------------------
// Batched shading: one launch shades the current instance segment of many
// independent command streams.  Each item is one (stream, pass, segment)
// with its own VRAM, records and bins; its work is cut into warp units
// (sub-tile, warp) -- 2 * 2^ns_log2 units per sub-tile, of which a
// single-sampled tile uses the first two -- that persistent warps take from a
// global counter, so streams of very different sizes share the GPU without
// a tail per stream.
struct ShadeItem
{
	PassParams P;
	DevInstance I;
	const uint32_t *masks, *summary, *flags;
	uint32_t ns_log2, aa;
	uint32_t unit_base, units;
};

// Sample counts the batched kernel shades itself (1x, 2x, 4x instances).
constexpr uint32_t BATCH_MAX_NS_LOG2 = 2;

// Separate functions per variant keep each variant's register allocation
// its own inside the batched kernel.
template <int NS, bool SS, bool AA>
__device__ __noinline__ void shade_subtile_call(const PassParams &P, const DevInstance &I, const uint32_t *sub_masks,
                                                const uint32_t *sub_summary, uint32_t sub, uint32_t t)
{
	shade_subtile<NS, SS, AA>(P, I, sub_masks, sub_summary, sub, t);
}

template <int BLOCK>
__global__ void __launch_bounds__(BLOCK, 1024 / BLOCK) batch_shade_kernel(const ShadeItem *items, uint32_t n_items,
                                                                         uint32_t total_units, uint32_t *counter)
{
	constexpr int WARPS = BLOCK / 32;
	__shared__ PassParams sP[WARPS];
	__shared__ DevInstance sI[WARPS];
	const uint32_t warp = threadIdx.x >> 5, lane = threadIdx.x & 31u;
	uint32_t loaded = 0xffffffffu;
	for (;;)
	{
		uint32_t unit = 0;
		if (lane == 0)
			unit = atomicAdd(counter, 1u);
		unit = __shfl_sync(0xffffffffu, unit, 0);
		if (unit >= total_units)
			break;
		uint32_t lo = 0, hi = n_items - 1;
		while (lo < hi)
		{
			uint32_t mid = (lo + hi + 1u) >> 1;
			if (items[mid].unit_base <= unit)
				lo = mid;
			else
				hi = mid - 1u;
		}
		const ShadeItem &it = items[lo];
		if (lo != loaded)
		{
			// Item parameters into this warp's shared slot.
			__syncwarp();
			const uint32_t *srcP = reinterpret_cast<const uint32_t *>(&it.P);
			uint32_t *dstP = reinterpret_cast<uint32_t *>(&sP[warp]);
			for (uint32_t k = lane; k < sizeof(PassParams) / 4; k += 32u)
				dstP[k] = srcP[k];
			const uint32_t *srcI = reinterpret_cast<const uint32_t *>(&it.I);
			uint32_t *dstI = reinterpret_cast<uint32_t *>(&sI[warp]);
			for (uint32_t k = lane; k < sizeof(DevInstance) / 4; k += 32u)
				dstI[k] = srcI[k];
			__syncwarp();
			loaded = lo;
		}
		const PassParams &P = sP[warp];
		const DevInstance &I = sI[warp];
		const uint32_t local = unit - it.unit_base;
		const uint32_t per_sub = 2u << it.ns_log2;
		const uint32_t sub = local / per_sub, w = local % per_sub;
		const uint32_t mode = subtile_mode(P, I, it.flags, sub);
		if (mode == 0)
			continue;
		const uint32_t ns_log2 = mode == 2 ? it.ns_log2 : 0u;
		if (w >= (2u << ns_log2))
			continue;
		const uint32_t t = w * 32u + lane;
		const bool aa = it.aa != 0;
		switch (ns_log2)
		{
		case 0:
			if (aa) shade_subtile_call<1, false, true>(P, I, it.masks, it.summary, sub, t);
			else shade_subtile_call<1, false, false>(P, I, it.masks, it.summary, sub, t);
			break;
		case 1:
			if (aa) shade_subtile_call<2, true, true>(P, I, it.masks, it.summary, sub, t);
			else shade_subtile_call<2, true, false>(P, I, it.masks, it.summary, sub, t);
			break;
		default:
			if (aa) shade_subtile_call<4, true, true>(P, I, it.masks, it.summary, sub, t);
			else shade_subtile_call<4, true, false>(P, I, it.masks, it.summary, sub, t);
			break;
		}
	}
}

// ---------------------------------------------------------------------------
// CRTC circuit read-out (sample_circuit.frag:98-148).  One thread per output
// texel; a 2x2 high-resolution read-out averages the sample planes of the
// quad position in float, in plane order, then converts to unorm8.
__device__ __forceinline__ uint32_t circuit_payload(const uint8_t *vram, uint32_t psm, uint32_t addr, uint32_t plane)
{
	if (psm_is_16bit(psm))
	{
		uint16_t v = reinterpret_cast<const uint16_t *>(vram)[addr + plane * (VRAM_SIZE / 2)];
		return rgba16_to_rgba32(v, 0, 0x0, 0xff);
	}
	uint32_t v = reinterpret_cast<const uint32_t *>(vram)[addr + plane * (VRAM_SIZE / 4)];
	if (psm != PSMCT32)
		v = (v & ~0xff000000u) | 0x80000000u;
	return v;
}

__global__ void __launch_bounds__(256) circuit_kernel(pgs_circuit_params C, const uint8_t *vram, const float *unorm_lut,
                                                      uint32_t *dst)
{
	const uint32_t x = blockIdx.x * 32u + (threadIdx.x & 31u), y = blockIdx.y * 8u + (threadIdx.x >> 5);
	if (x >= C.width || y >= C.height)
		return;
	uint32_t out = 0;
	if (x < C.valid_width && y < C.valid_height)
	{
		const uint32_t sx = C.super_samples >= 4 ? x >> 1 : x, sy = C.super_samples >= 4 ? y >> 1 : y;
		const uint32_t cx = sx + C.dbx, cy = sy * C.phase_stride + C.dby + C.phase;
		const uint32_t addr = swizzle_address(cx, cy, C.fbp * BLOCKS_PER_PAGE, C.fbw, C.psm);
		bool resolve = false;
		if (C.super_samples >= 4)
		{
			if (psm_is_16bit(C.psm))
				resolve = reinterpret_cast<const uint16_t *>(vram)[addr + VRAM_SIZE / 2] == 0xffffu;
			else
			{
				uint32_t ref = reinterpret_cast<const uint32_t *>(vram)[addr + VRAM_SIZE / 4];
				resolve = C.psm != PSMCT32 ? (ref & 0xffffffu) == 0xffffffu : ref == 0xffffffffu;
			}
		}
		if (!resolve)
			out = circuit_payload(vram, C.psm, addr, 0);
		else
		{
			const uint32_t n = C.super_samples / 4;
			const uint32_t quad = C.super_samples != 8 ? (y & 1u) + (x & 1u) * 2u : (x & 1u) + (y & 1u) * 2u;
			const uint32_t base = 2u + n * quad;
			float v[4] = { 0.0f, 0.0f, 0.0f, 0.0f };
			for (uint32_t i = 0; i < n; i++)
			{
				uint32_t c = circuit_payload(vram, C.psm, addr, base + i);
				#pragma unroll
				for (int k = 0; k < 4; k++)
					v[k] = fadd(v[k], unorm_lut[(c >> (8 * k)) & 0xffu]);
			}
			const float fn = float(n);
			out = pack_unorm(__fdiv_rn(v[0], fn), __fdiv_rn(v[1], fn), __fdiv_rn(v[2], fn), __fdiv_rn(v[3], fn));
		}
	}
	dst[size_t(y) * C.width + x] = out;
}

// ---------------------------------------------------------------------------
// vsync output merge (GSRenderer::vsync, gs/gs_renderer.cpp:4738-4866): the
// circuits are stretched into their CRTC viewports over a BGCOLOR clear.
// The stretch is bilinear with 8-bit sub-texel positions, clamped to the
// edge: texel coordinate = ((2 d + 1) * src / (2 * dst)) - 1/2 in 1/256 units,
// exact texels when source and viewport have the same size.  Blends are
// integer: (c * a + d * (255 - a)) / 255 rounded to nearest, alpha from the
// source (blend factors SRC/CONSTANT_ALPHA, ONE/ZERO on alpha).

__device__ __forceinline__ uint32_t stretch_sample(const uint32_t *img, uint32_t iw, uint32_t ih, int32_t dx, int32_t dy,
                                                   uint32_t vw, uint32_t vh)
{
	const int64_t fx = (int64_t(2 * dx + 1) * iw * 256) / (2 * int64_t(vw)) - 128;
	const int64_t fy = (int64_t(2 * dy + 1) * ih * 256) / (2 * int64_t(vh)) - 128;
	const int32_t x0 = int32_t(fx >> 8), y0 = int32_t(fy >> 8);
	const uint32_t wx = uint32_t(fx & 255), wy = uint32_t(fy & 255);
	const int32_t xa = min(max(x0, 0), int32_t(iw) - 1), xb = min(max(x0 + 1, 0), int32_t(iw) - 1);
	const int32_t ya = min(max(y0, 0), int32_t(ih) - 1), yb = min(max(y0 + 1, 0), int32_t(ih) - 1);
	const uint32_t c00 = img[size_t(ya) * iw + xa], c10 = img[size_t(ya) * iw + xb];
	const uint32_t c01 = img[size_t(yb) * iw + xa], c11 = img[size_t(yb) * iw + xb];
	const uint32_t w00 = (256u - wx) * (256u - wy), w10 = wx * (256u - wy), w01 = (256u - wx) * wy, w11 = wx * wy;
	uint32_t out = 0;
	#pragma unroll
	for (int k = 0; k < 4; k++)
	{
		const int sh = 8 * k;
		uint32_t acc = w00 * ((c00 >> sh) & 255u) + w10 * ((c10 >> sh) & 255u) + w01 * ((c01 >> sh) & 255u) +
		               w11 * ((c11 >> sh) & 255u);
		out |= ((acc + 32768u) >> 16) << sh;
	}
	return out;
}

__device__ __forceinline__ uint32_t blend255(uint32_t s, uint32_t d, uint32_t a)
{
	const uint32_t v = s * a + d * (255u - a);
	const uint32_t q = v / 255u, r = v % 255u;
	return q + (2u * r > 255u ? 1u : 0u);
}

__global__ void __launch_bounds__(256) merge_kernel(pgs_merge_params M, const uint32_t *c1, const uint32_t *c2, uint32_t *dst)
{
	const uint32_t x = blockIdx.x * 32u + (threadIdx.x & 31u), y = blockIdx.y * 8u + (threadIdx.x >> 5);
	if (x >= M.width || y >= M.height)
		return;
	uint32_t color = M.bgcolor & 0xffffffu;
	const int32_t ix = int32_t(x), iy = int32_t(y);
	if (M.draw_circuit2 && M.rect_w[1] && M.rect_h[1] && ix >= M.rect_x[1] && ix < M.rect_x[1] + int32_t(M.rect_w[1]) &&
	    iy >= M.rect_y[1] && iy < M.rect_y[1] + int32_t(M.rect_h[1]))
		color = stretch_sample(c2, M.circuit[1].width, M.circuit[1].height, ix - M.rect_x[1], iy - M.rect_y[1],
		                       M.rect_w[1], M.rect_h[1]);
	if (M.draw_circuit1 && M.rect_w[0] && M.rect_h[0] && ix >= M.rect_x[0] && ix < M.rect_x[0] + int32_t(M.rect_w[0]) &&
	    iy >= M.rect_y[0] && iy < M.rect_y[0] + int32_t(M.rect_h[0]))
	{
		const uint32_t s = stretch_sample(c1, M.circuit[0].width, M.circuit[0].height, ix - M.rect_x[0],
		                                  iy - M.rect_y[0], M.rect_w[0], M.rect_h[0]);
		if (M.blend == 0)
			color = s;
		else
		{
			const uint32_t a = M.blend == 1 ? M.alp : (s >> 24);
			uint32_t out = s & 0xff000000u;
			#pragma unroll
			for (int k = 0; k < 3; k++)
				out |= blend255((s >> (8 * k)) & 255u, (color >> (8 * k)) & 255u, a) << (8 * k);
			color = out;
		}
	}
	dst[size_t(y) * M.width + x] = color;
}

// EXTWRITE (extwrite.comp:37-98): the merged image or a circuit written back
// into VRAM as CT32 at (WDX, WDY) of EXBP / EXBW, nearest texel at
// uv = base + id * scale, optionally converted to Y / YCbCr / alpha.  Float
// expressions are evaluated left to right, one rounding per operation.
__global__ void __launch_bounds__(256) extwrite_kernel(pgs_merge_params M, const uint32_t *src, uint32_t sw, uint32_t sh,
                                                       const float *unorm_lut, uint8_t *vram, uint32_t invalidate_ss)
{
	const uint32_t gx = blockIdx.x * 32u + (threadIdx.x & 31u), gy = blockIdx.y * 8u + (threadIdx.x >> 5);
	if (gx >= M.ext_width || gy >= M.ext_height)
		return;
	const float u = fadd(M.ext_uv_base[0], fmul(__uint2float_rn(gx), M.ext_uv_scale[0]));
	const float v = fadd(M.ext_uv_base[1], fmul(__uint2float_rn(gy), M.ext_uv_scale[1]));
	const int32_t tx = min(max(int32_t(floorf(fmul(u, __uint2float_rn(sw)))), 0), int32_t(sw) - 1);
	const int32_t ty = min(max(int32_t(floorf(fmul(v, __uint2float_rn(sh)))), 0), int32_t(sh) - 1);
	const uint32_t c = src[size_t(ty) * sw + tx];
	const float r = unorm_lut[c & 255u], g = unorm_lut[(c >> 8) & 255u], b = unorm_lut[(c >> 16) & 255u];
	const float a = unorm_lut[c >> 24];
	const float ey = fadd(fadd(fmul(0.587f, g), fmul(0.114f, b)), fmul(0.299f, r));
	const float ecb = fsub(fadd(fmul(-0.311f, g), fmul(0.500f, b)), fmul(0.169f, r));
	const float ecr = fadd(fsub(fmul(-0.419f, g), fmul(0.081f, b)), fmul(0.500f, r));
	const float Y = __fdiv_rn(fadd(fmul(219.0f, ey), 16.0f), 255.0f);
	const float Cb = __fdiv_rn(fadd(fmul(224.0f, ecb), 128.0f), 255.0f);
	const float Cr = __fdiv_rn(fadd(fmul(224.0f, ecr), 128.0f), 255.0f);
	float o[4];
	switch (M.ext_emodc)
	{
	case 0: o[0] = r; o[1] = g; o[2] = b; break;
	case 1: o[0] = Y; o[1] = Y; o[2] = Y; break;
	case 2: o[0] = Y; o[1] = Cb; o[2] = Cr; break;
	default: o[0] = a; o[1] = a; o[2] = a; break;
	}
	switch (M.ext_emoda)
	{
	case 0: o[3] = a; break;
	case 1: o[3] = Y; break;
	case 2: o[3] = fmul(0.5f, Y); break;
	default: o[3] = 0.0f; break;
	}
	const uint32_t addr = swizzle_address(gx + M.ext_wdx, gy + M.ext_wdy, M.ext_exbp, M.ext_exbw, PSMCT32);
	reinterpret_cast<uint32_t *>(vram)[addr] = pack_unorm(o[0], o[1], o[2], o[3]);
	if (invalidate_ss)
		reinterpret_cast<uint32_t *>(vram)[addr + VRAM_SIZE / 4] = 0;
}

// FastMAD deinterlace (weave.frag): lines of the current field pass through;
// the others pick between the previous field (weave) and the average of the
// current field's neighbours (bob) by the local luma difference, with
// smoothstep(0.04, 0.06, diff) and mix() evaluated left to right.
__device__ __forceinline__ float luma_diff(const float *lut, uint32_t a, uint32_t b)
{
	const float dr = fsub(lut[a & 255u], lut[b & 255u]);
	const float dg = fsub(lut[(a >> 8) & 255u], lut[(b >> 8) & 255u]);
	const float db = fsub(lut[(a >> 16) & 255u], lut[(b >> 16) & 255u]);
	return fabsf(fadd(fadd(fmul(dr, 0.299f), fmul(dg, 0.587f)), fmul(db, 0.114f)));
}

__global__ void __launch_bounds__(256) weave_kernel(const uint32_t *f0, const uint32_t *f1, const uint32_t *f2,
                                                    const uint32_t *f3, uint32_t width, uint32_t field_height,
                                                    uint32_t phase, const float *lut, uint32_t *dst)
{
	const uint32_t x = blockIdx.x * 32u + (threadIdx.x & 31u), y = blockIdx.y * 8u + (threadIdx.x >> 5);
	const uint32_t height = 2u * field_height;
	if (x >= width || y >= height)
		return;
	uint32_t out;
	if ((y & 1u) == phase)
		out = f0[size_t(y >> 1) * width + x];
	else if (y == 0 || y == height - 1u)
		out = f1[size_t(y >> 1) * width + x];
	else
	{
		const uint32_t up = (y - 1u) >> 1;
		const uint32_t cur0 = f0[size_t(up) * width + x], cur1 = f0[size_t(up + 1u) * width + x];
		const uint32_t prev0 = f2[size_t(up) * width + x], prev1 = f2[size_t(up + 1u) * width + x];
		const uint32_t fld1 = f1[size_t(y >> 1) * width + x], fld3 = f3[size_t(y >> 1) * width + x];
		const float mh = luma_diff(lut, cur0, prev0), ml = luma_diff(lut, cur1, prev1), mc = luma_diff(lut, fld1, fld3);
		const float diff = fmaxf(fminf(mh, ml), mc);
		const float tt = fminf(fmaxf(__fdiv_rn(fsub(diff, 0.04f), fsub(0.06f, 0.04f)), 0.0f), 1.0f);
		const float bob = fmul(fmul(tt, tt), fsub(3.0f, fmul(2.0f, tt)));
		float o[3];
		#pragma unroll
		for (int k = 0; k < 3; k++)
		{
			const float avg = fmul(0.5f, fadd(lut[(cur0 >> (8 * k)) & 255u], lut[(cur1 >> (8 * k)) & 255u]));
			o[k] = fadd(fmul(lut[(fld1 >> (8 * k)) & 255u], fsub(1.0f, bob)), fmul(avg, bob));
		}
		out = pack_unorm(o[0], o[1], o[2], 1.0f);
	}
	dst[size_t(y) * width + x] = out;
}

// ---------------------------------------------------------------------------
// K4: VRAM transfers.
struct CopyParams
{
	uint32_t sbp, sbw, spsm, dbp, dbw, dpsm;
	uint32_t ssax, ssay, dsax, dsay, width, height;
	uint32_t xdir;
	uint64_t host_size, host_offset_qwords;
	const uint8_t *host;      // device copy of the HWREG payload
	const uint8_t *src_vram;  // snapshot for local->local
	uint32_t invalidate_ss;
};

__device__ __forceinline__ void write_pixel(uint8_t *vram, uint32_t psm, uint32_t addr, uint32_t data, bool inv)
{
	uint32_t *v32 = reinterpret_cast<uint32_t *>(vram);
	uint16_t *v16 = reinterpret_cast<uint16_t *>(vram);
	const uint32_t V32 = VRAM_SIZE / 4, V16 = VRAM_SIZE / 2;
	switch (psm)
	{
	case PSMCT24: case PSMZ24:
	{
		uint8_t *b = vram + size_t(addr) * 4u;
		b[0] = uint8_t(data); b[1] = uint8_t(data >> 8); b[2] = uint8_t(data >> 16);
		if (inv) { uint8_t *r = b + VRAM_SIZE; r[0] = 0; r[1] = 0; r[2] = 0; }
		break;
	}
	case PSMCT16: case PSMCT16S: case PSMZ16: case PSMZ16S:
		v16[addr] = uint16_t(data);
		if (inv) v16[addr + V16] = 0;
		break;
	case PSMT8:
		vram[addr] = uint8_t(data);
		if (inv) vram[addr + VRAM_SIZE] = 0;
		break;
	case PSMT8H:
		vram[addr * 4u + 3u] = uint8_t(data);
		if (inv) vram[addr * 4u + 3u + VRAM_SIZE] = 0;
		break;
	case PSMT4:
	{
		uint32_t word = addr >> 3, sh = 4u * (addr & 7u);
		atomicAnd(&v32[word], ~(0xfu << sh));
		atomicOr(&v32[word], (data & 0xfu) << sh);
		if (inv) atomicAnd(&v32[word + V32], ~(0xfu << sh));
		break;
	}
	case PSMT4HL: case PSMT4HH:
	{
		uint32_t sh = psm == PSMT4HL ? 24u : 28u;
		v32[addr] = (v32[addr] & ~(0xfu << sh)) | ((data & 0xfu) << sh);
		if (inv) v32[addr + V32] &= ~(0xfu << sh);
		break;
	}
	default:
		v32[addr] = data;
		if (inv) v32[addr + V32] = 0;
		break;
	}
}

__device__ __forceinline__ uint32_t read_pixel(const uint8_t *vram, uint32_t psm, uint32_t a)
{
	const uint32_t *v32 = reinterpret_cast<const uint32_t *>(vram);
	const uint16_t *v16 = reinterpret_cast<const uint16_t *>(vram);
	if (psm_is_16bit(psm)) return v16[a];
	if (psm == PSMT8) return vram[a];
	if (psm == PSMT8H) return vram[4u * a + 3u];
	if (psm == PSMT4) return (uint32_t(vram[a >> 1]) >> ((a & 1u) * 4u)) & 15u;
	if (psm == PSMT4HL) return (v32[a] >> 24) & 15u;
	if (psm == PSMT4HH) return v32[a] >> 28;
	return v32[a];
}

__device__ __forceinline__ void upload_pixel(const CopyParams &C, uint8_t *vram, uint32_t x, uint32_t y)
{
	if (x >= C.width || y >= C.height)
		return;
	uint32_t eff_stride = C.dbw;
	if (C.dpsm == PSMT4 || C.dpsm == PSMT8)
		eff_stride &= ~1u;
	if (x >= eff_stride * 64u)
	{
		Layout L = psm_layout(C.dpsm);
		uint32_t last = (C.dsay + C.height - 1u) >> L.ph, cur = (C.dsay + y) >> L.ph;
		if (last != cur)
			return;
	}
	uint32_t dx = (x + C.dsax) & 2047u, dy = (y + C.dsay) & 2047u;
	uint32_t data;
	if (C.xdir == HOST_TO_LOCAL)
	{
		uint64_t sa = uint64_t(y) * C.width + x;
		uint32_t b = psm_bits_per_pixel(C.dpsm);
		uint64_t factor = (b == 32 || b == 24) ? 2 : (b == 16 ? 4 : (b == 8 ? 8 : 16));
		uint64_t avail = b == 32 ? C.host_size / 4 : (b == 24 ? C.host_size / 3 : (b == 16 ? C.host_size / 2 : (b == 8 ? C.host_size : 2 * C.host_size)));
		if (sa * factor < C.host_offset_qwords || sa >= avail)
			return;
		// The payload starts 256-byte aligned: a warp's 32 consecutive pixels
		// read one contiguous span, with one load of the pixel's width each.
		const uint8_t *h = C.host;
		if (b == 24) data = uint32_t(h[3 * sa]) | (uint32_t(h[3 * sa + 1]) << 8) | (uint32_t(h[3 * sa + 2]) << 16);
		else if (b == 16) data = reinterpret_cast<const uint16_t *>(h)[sa];
		else if (b == 8) data = h[sa];
		else if (b == 4) data = (uint32_t(h[sa >> 1]) >> ((sa & 1) * 4)) & 15u;
		else data = reinterpret_cast<const uint32_t *>(h)[sa];
	}
	else
	{
		uint32_t sx = (x + C.ssax) & 2047u, sy = (y + C.ssay) & 2047u;
		data = read_pixel(C.src_vram, C.spsm, swizzle_address(sx, sy, C.sbp, C.sbw, C.spsm));
	}
	write_pixel(vram, C.dpsm, swizzle_address(dx, dy, C.dbp, C.dbw, C.dpsm), data, C.invalidate_ss != 0);
}

__global__ void __launch_bounds__(256) upload_kernel(CopyParams C, uint8_t *vram)
{
	upload_pixel(C, vram, blockIdx.x * 32u + (threadIdx.x & 31u), blockIdx.y * 8u + (threadIdx.x >> 5));
}

// Consecutive host->local uploads whose destination blocks do not overlap, in
// one launch: the order among them cannot change VRAM.  Blocks of 32 x 8
// pixels are dealt out to the uploads by block_start.
constexpr uint32_t UPLOAD_BATCH_MAX = 16;
struct UploadBatch
{
	CopyParams c[UPLOAD_BATCH_MAX];
	uint32_t block_start[UPLOAD_BATCH_MAX + 1];
	uint32_t count;
};

__global__ void __launch_bounds__(256) upload_batch_kernel(UploadBatch B, uint8_t *vram)
{
	uint32_t i = 0;
	while (i + 1u < B.count && blockIdx.x >= B.block_start[i + 1])
		i++;
	const CopyParams &C = B.c[i];
	const uint32_t local = blockIdx.x - B.block_start[i], bw = (C.width + 31u) / 32u;
	upload_pixel(C, vram, (local % bw) * 32u + (threadIdx.x & 31u), (local / bw) * 8u + (threadIdx.x >> 5));
}

// LOCAL->HOST read-out of a rectangle of plane 0 into linear bytes
// (vram_readback, gs/gs_util.hpp:50-110): pixels in row order at their host
// size (4, 3, 2 or 1 bytes).  Each thread packs 16 consecutive output bytes
// and writes them as one 16-byte store where the output allows.
struct ReadbackParams
{
	uint32_t sbp, sbw, spsm, ssax, ssay, width, height, bytes_per_pixel;
	uint64_t size; // output bytes
};

// Byte k of the pixel at word/halfword/byte address a.
__device__ __forceinline__ uint32_t readback_fetch(uint32_t spsm, const uint8_t *vram, uint32_t a, uint32_t k)
{
	switch (spsm)
	{
	case PSMCT16: case PSMCT16S: case PSMZ16: case PSMZ16S: return vram[2u * a + k];
	case PSMT8: return vram[a];
	case PSMT8H: return vram[4u * a + 3u];
	default: return vram[4u * a + k];
	}
}

__global__ void __launch_bounds__(256) readback_kernel(ReadbackParams R, const uint8_t *vram, uint8_t *out)
{
	const uint64_t first = (uint64_t(blockIdx.x) * blockDim.x + threadIdx.x) * 16u;
	if (first >= R.size)
		return;
	const uint32_t B = R.bytes_per_pixel;
	const uint64_t i = first / B;
	uint32_t k = uint32_t(first - i * B);
	uint32_t x = uint32_t(i % R.width), y = uint32_t(i / R.width);
	uint32_t a = swizzle_address((x + R.ssax) & 2047u, (y + R.ssay) & 2047u, R.sbp, R.sbw, R.spsm);
	auto next = [&]() {
		const uint32_t v = readback_fetch(R.spsm, vram, a, k);
		if (++k == B)
		{
			k = 0;
			if (++x == R.width)
			{
				x = 0;
				y++;
			}
			a = swizzle_address((x + R.ssax) & 2047u, (y + R.ssay) & 2047u, R.sbp, R.sbw, R.spsm);
		}
		return v;
	};
	if (first + 16u <= R.size)
	{
		uint32_t w[4];
		#pragma unroll
		for (int q = 0; q < 4; q++)
		{
			uint32_t v = 0;
			#pragma unroll
			for (int b = 0; b < 4; b++)
				v |= next() << (8 * b);
			w[q] = v;
		}
		*reinterpret_cast<uint4 *>(out + first) = make_uint4(w[0], w[1], w[2], w[3]);
	}
	else
		for (uint64_t b = first; b < R.size; b++)
			out[b] = uint8_t(next());
}

// ---------------------------------------------------------------------------
// K6: CLUT load into a new ring instance.
struct ClutParams
{
	uint32_t psm, cbp, cpsm, csm, csa, cbw, cou, cov;
	float csm2_x_scale;
	uint32_t csm2_x_bias;
	uint32_t base_instance, instance;
};

// One CLUT load applied to the 512 entries in tmp (256 threads).
__device__ __forceinline__ void clut_apply(const ClutParams &C, const uint8_t *vram, uint16_t *tmp, uint32_t lane)
{
	bool index4 = C.psm == PSMT4 || C.psm == PSMT4HH || C.psm == PSMT4HL;
	bool active;
	uint32_t wc = lane + C.csa * 16u, rc = lane;
	if (index4)
		active = lane < 16u;
	else if (C.csm == 0)
	{
		uint32_t csa_count = C.cpsm == PSMCT32 ? 16u : 32u;
		active = lane < (csa_count - C.csa) * 16u;
		rc += C.csa * 16u;
	}
	else
		active = true;
	if (active)
	{
		uint32_t cx, cy;
		if (C.csm)
		{
			cx = uint32_t(fadd(fmul(float(rc), C.csm2_x_scale), 1.0f / 256.0f)) + C.csm2_x_bias + C.cou * 16u;
			cy = C.cov;
		}
		else
		{
			cx = (rc & 7u) | (((rc >> 4) & 1u) << 3);
			cy = ((rc >> 3) & 1u) | (((rc >> 5) & 7u) << 1);
		}
		if (C.cpsm == PSMCT32)
		{
			uint32_t v = reinterpret_cast<const uint32_t *>(vram)[swizzle_address(cx, cy, C.cbp, C.cbw, PSMCT32)];
			if (wc < 512u) tmp[wc] = uint16_t(v);
			if (wc + 256u < 512u) tmp[wc + 256u] = uint16_t(v >> 16);
		}
		else
		{
			uint32_t v = reinterpret_cast<const uint16_t *>(vram)[swizzle_address(cx, cy, C.cbp, C.cbw, C.cpsm)];
			if (wc < 512u) tmp[wc] = uint16_t(v);
		}
	}
}

__global__ void __launch_bounds__(256) clut_kernel(ClutParams C, const uint8_t *vram, uint16_t *clut)
{
	__shared__ uint16_t tmp[512];
	uint32_t lane = threadIdx.x;
	tmp[lane] = clut[size_t(C.base_instance) * 512u + lane];
	tmp[lane + 256u] = clut[size_t(C.base_instance) * 512u + lane + 256u];
	__syncthreads();
	clut_apply(C, vram, tmp, lane);
	__syncthreads();
	clut[size_t(C.instance) * 512u + lane] = tmp[lane];
	clut[size_t(C.instance) * 512u + lane + 256u] = tmp[lane + 256u];
}

// A chain of consecutive CLUT loads (each one's base is the previous one's
// instance) in one launch: block k starts from the first load's base and
// applies loads 0..k, so it writes the instance load k would have written.
// VRAM does not change between the loads, and no load of the chain writes
// the first load's base.
constexpr uint32_t CLUT_BATCH_MAX = 16;
struct ClutBatch
{
	ClutParams c[CLUT_BATCH_MAX];
	uint32_t count;
};

__global__ void __launch_bounds__(256) clut_batch_kernel(ClutBatch B, const uint8_t *vram, uint16_t *clut)
{
	__shared__ uint16_t tmp[512];
	const uint32_t lane = threadIdx.x, k = blockIdx.x;
	// An 8-bit CT32 load at CSA 0 rewrites all 512 entries: start from the
	// last one at or before k.
	uint32_t j0 = 0;
	for (uint32_t j = k + 1u; j-- > 0u;)
	{
		const ClutParams &c = B.c[j];
		if ((c.psm == PSMT8 || c.psm == PSMT8H) && c.csm == 0 && c.cpsm == PSMCT32 && c.csa == 0)
		{
			j0 = j;
			break;
		}
	}
	const uint32_t base = B.c[0].base_instance;
	tmp[lane] = clut[size_t(base) * 512u + lane];
	tmp[lane + 256u] = clut[size_t(base) * 512u + lane + 256u];
	__syncthreads();
	for (uint32_t j = j0; j <= k; j++)
	{
		clut_apply(B.c[j], vram, tmp, lane);
		__syncthreads();
	}
	clut[size_t(B.c[k].instance) * 512u + lane] = tmp[lane];
	clut[size_t(B.c[k].instance) * 512u + lane + 256u] = tmp[lane + 256u];
}
} // namespace pgs
