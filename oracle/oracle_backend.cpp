// oracle_backend.cpp -- CPU restatement of the reference's GPU backend.
//
// TEST INFRASTRUCTURE ONLY.  This file is the checker that the CUDA backend is
// compared against; it is never linked into the product library.  It
// implements pgs_backend_ops with plain sequential C++:
//
//   triangle_setup   gs/shaders/triangle_setup.comp:127-873
//   binning          gs/shaders/binning.comp:74-313 (membership, order and the
//                    per-tile super-sampling decision)
//   shading          gs/shaders/ubershader.comp:435-1816, one pixel-sample at a
//                    time, primitives in ascending index order
//   transfers        gs/shaders/vram_copy.comp:261-614
//   CLUT loads       gs/shaders/clut_write.comp:46-156
//
// Floating-point steps that the reference leaves to the Vulkan driver are
// pinned to single IEEE operations with no contraction (the file is built
// with -ffp-contract=off):
//  * unpackUnorm4x8(c) = float(c) / 255.0f, packUnorm4x8(x) = roundEven(clamp(x,0,1) * 255).
//  * Expressions without `precise` are evaluated left to right, one rounding
//    per operation (no FMA).
//  * The hardware sampler is replaced by exact integer filtering: the snapped
//    coordinate k = floor(uv * 16 + 1/64) selects texel k >> 4 (nearest) or
//    texels (k - 8) >> 4 and +1 with weight ((k - 8) & 15) / 16 (linear); the
//    result is roundEven(sum(w_x * w_y * c) / 256).
//  * Texels are read from swizzled VRAM and the CLUT directly (upload.comp's
//    decode, gs/shaders/upload.comp:76-229), not from a cached image.
#include "pgs.h"

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <new>
#include <vector>

namespace oracle
{
// ---------------------------------------------------------------------------
// Formats and swizzle (gs/shaders/swizzle_utils.h:93-522).
enum : uint32_t
{
	CT32 = 0x00, CT24 = 0x01, CT16 = 0x02, CT16S = 0x0a, T8 = 0x13, T4 = 0x14, T8H = 0x1b,
	T4HL = 0x24, T4HH = 0x2c, Z32 = 0x30, Z24 = 0x31, Z16 = 0x32, Z16S = 0x3a
};

static const uint32_t VRAM = 4u * 1024u * 1024u;

static bool is16(uint32_t p) { return p == CT16 || p == CT16S || p == Z16 || p == Z16S; }
static bool is24(uint32_t p) { return p == CT24 || p == Z24; }
static bool is32(uint32_t p) { return p == CT32 || p == Z32; }

static uint32_t bpp(uint32_t p)
{
	if (is24(p)) return 24;
	if (is16(p)) return 16;
	if (p == T8 || p == T8H) return 8;
	if (p == T4 || p == T4HL || p == T4HH) return 4;
	return 32;
}

struct Geo { uint32_t page_w, page_h, block_w, block_h, column_h; };

static Geo geometry(uint32_t p)
{
	if (is16(p)) return { 64, 64, 16, 8, 2 };
	if (p == T8) return { 128, 64, 16, 16, 4 };
	if (p == T4) return { 128, 128, 32, 16, 4 };
	return { 64, 32, 8, 8, 2 };
}

static uint32_t swizzle(uint32_t x, uint32_t y, uint32_t base, uint32_t stride, uint32_t fmt)
{
	Geo g = geometry(fmt);
	if (fmt == T4 || fmt == T8)
		stride >>= 1;
	uint32_t page = (y / g.page_h) * stride + (x / g.page_w);
	uint32_t bx = (x % g.page_w) / g.block_w;
	uint32_t by = (y % g.page_h) / g.block_h;
	uint32_t col = (y % g.block_h) / g.column_h;
	uint32_t px = x % g.block_w;
	uint32_t py = y % g.column_h;
	uint32_t b32 = (bx & 1) | ((by & 1) << 1) | ((bx & 2) << 1) | ((by & 2) << 2) | ((bx & 4) << 2);
	uint32_t b16 = (by & 1) | ((bx & 1) << 1) | ((by & 2) << 1) | ((bx & 2) << 2) | ((by & 4) << 2);
	uint32_t b16s = (by & 1) | ((bx & 1) << 1) | (by & 4) | ((by & 2) << 2) | ((bx & 2) << 3);
	uint32_t p32 = (px & 1) | ((py & 1) << 1) | ((px & 2) << 1) | ((px & 4) << 1);
	uint32_t p16 = ((px & 8) >> 3) | ((px & 1) << 1) | ((py & 1) << 2) | ((px & 2) << 2) | ((px & 4) << 2);
	uint32_t head = page * 8192u + col * 64u;

	switch (fmt)
	{
	case Z32: case Z24:
		return ((head + ((b32 + base) ^ 0x18u) * 256u + p32 * 4u) & (VRAM - 1)) >> 2;
	case CT16: return ((head + (b16 + base) * 256u + p16 * 2u) & (VRAM - 1)) >> 1;
	case Z16: return ((head + ((b16 + base) ^ 0x18u) * 256u + p16 * 2u) & (VRAM - 1)) >> 1;
	case CT16S: return ((head + (b16s + base) * 256u + p16 * 2u) & (VRAM - 1)) >> 1;
	case Z16S: return ((head + ((b16s + base) ^ 0x18u) * 256u + p16 * 2u) & (VRAM - 1)) >> 1;
	case T8:
	{
		uint32_t p = ((py & 2) >> 1) | ((px & 8) >> 2) | ((px & 1) << 2) | ((py & 1) << 3) | ((px & 2) << 3) |
		             ((((px & 4) << 3) ^ ((py & 2) << 4)) ^ ((col & 1) << 5));
		return (head + (b32 + base) * 256u + p) & (VRAM - 1);
	}
	case T4:
	{
		uint32_t p = ((py & 2) >> 1) | ((px & 8) >> 2) | ((px & 16) >> 2) | ((px & 1) << 3) | ((py & 1) << 4) |
		             ((px & 2) << 4) | ((((px & 4) << 4) ^ ((py & 2) << 5)) ^ ((col & 1) << 6));
		return (((head + (b16 + base) * 256u) << 1) + p) & ((VRAM << 1) - 1);
	}
	default:
		return ((head + (b32 + base) * 256u + p32 * 4u) & (VRAM - 1)) >> 2;
	}
}

// ---------------------------------------------------------------------------
// Helpers with GLSL semantics.
static uint32_t bfe(uint32_t v, int off, int bits) { return (v >> off) & ((bits >= 32) ? ~0u : ((1u << bits) - 1u)); }
static float u2f(uint32_t u) { float f; memcpy(&f, &u, 4); return f; }
static uint32_t f2u(float f) { uint32_t u; memcpy(&u, &f, 4); return u; }
static float round_even(float x) { return std::nearbyint(x); }
static int clz32(uint32_t b) { return b ? __builtin_clz(b) : 32; }
static uint32_t mulhi(uint32_t a, uint32_t b) { return uint32_t((uint64_t(a) * b) >> 32); }

static float unorm(uint32_t c, int ch) { return float((c >> (8 * ch)) & 0xffu) / 255.0f; }

static uint32_t pack_unorm(const float v[4])
{
	uint32_t r = 0;
	for (int i = 0; i < 4; i++)
	{
		float x = std::min(std::max(v[i], 0.0f), 1.0f);
		r |= uint32_t(round_even(x * 255.0f)) << (8 * i);
	}
	return r;
}

// 256-entry fixed-point reciprocal seed table (gs/gs_renderer.cpp:3602-3636).
static const uint8_t RCP_TAB[256] = {
	0xff, 0xfd, 0xfb, 0xf9, 0xf7, 0xf5, 0xf3, 0xf1, 0xf0, 0xee, 0xec, 0xea, 0xe8, 0xe6, 0xe5, 0xe3,
	0xe1, 0xdf, 0xdd, 0xdc, 0xda, 0xd8, 0xd7, 0xd5, 0xd3, 0xd2, 0xd0, 0xce, 0xcd, 0xcb, 0xc9, 0xc8,
	0xc6, 0xc5, 0xc3, 0xc2, 0xc0, 0xbf, 0xbd, 0xbc, 0xba, 0xb9, 0xb7, 0xb6, 0xb4, 0xb3, 0xb1, 0xb0,
	0xae, 0xad, 0xac, 0xaa, 0xa9, 0xa7, 0xa6, 0xa5, 0xa4, 0xa2, 0xa1, 0x9f, 0x9e, 0x9d, 0x9c, 0x9a,
	0x99, 0x98, 0x96, 0x95, 0x94, 0x93, 0x91, 0x90, 0x8f, 0x8e, 0x8c, 0x8b, 0x8a, 0x89, 0x88, 0x87,
	0x86, 0x84, 0x83, 0x82, 0x81, 0x80, 0x7f, 0x7e, 0x7c, 0x7b, 0x7a, 0x79, 0x78, 0x77, 0x76, 0x74,
	0x74, 0x73, 0x71, 0x71, 0x70, 0x6f, 0x6e, 0x6d, 0x6b, 0x6b, 0x6a, 0x68, 0x67, 0x67, 0x66, 0x65,
	0x64, 0x63, 0x62, 0x61, 0x60, 0x5f, 0x5e, 0x5d, 0x5c, 0x5b, 0x5b, 0x59, 0x58, 0x58, 0x56, 0x56,
	0x55, 0x54, 0x53, 0x52, 0x51, 0x51, 0x50, 0x4f, 0x4e, 0x4e, 0x4c, 0x4b, 0x4b, 0x4a, 0x48, 0x48,
	0x48, 0x46, 0x46, 0x45, 0x44, 0x43, 0x43, 0x42, 0x41, 0x40, 0x3f, 0x3f, 0x3e, 0x3d, 0x3c, 0x3b,
	0x3b, 0x3a, 0x39, 0x38, 0x38, 0x37, 0x36, 0x36, 0x35, 0x34, 0x34, 0x33, 0x32, 0x31, 0x30, 0x30,
	0x2f, 0x2e, 0x2e, 0x2d, 0x2d, 0x2c, 0x2b, 0x2a, 0x2a, 0x29, 0x28, 0x27, 0x27, 0x26, 0x26, 0x25,
	0x24, 0x23, 0x23, 0x22, 0x21, 0x21, 0x21, 0x20, 0x1f, 0x1f, 0x1e, 0x1d, 0x1d, 0x1c, 0x1c, 0x1b,
	0x1a, 0x19, 0x19, 0x19, 0x18, 0x17, 0x17, 0x16, 0x16, 0x15, 0x14, 0x13, 0x13, 0x12, 0x12, 0x11,
	0x11, 0x10, 0x0f, 0x0f, 0x0e, 0x0e, 0x0e, 0x0d, 0x0c, 0x0c, 0x0b, 0x0b, 0x0a, 0x0a, 0x09, 0x08,
	0x08, 0x07, 0x07, 0x07, 0x06, 0x05, 0x05, 0x04, 0x04, 0x03, 0x03, 0x02, 0x02, 0x01, 0x01, 0x01,
};

// rcp_fixed (gs/shaders/math_utils.h:27-61).
static float rcp_fixed(uint32_t b)
{
	int lz = clz32(b);
	uint32_t nb = b << lz;
	uint32_t idx = (nb >> 23) & 0xffu;
	uint32_t rcp = uint32_t(RCP_TAB[idx]) | 0x100u;
	uint32_t f = (rcp * rcp) << 14;
	uint32_t p = mulhi(f, nb);
	rcp = (rcp << 23) - p;
	rcp <<= 1;
	p = mulhi(rcp, nb);
	rcp = mulhi(rcp, 0u - p);
	rcp = (rcp + 64u) >> 7;
	rcp -= 1u << 23;
	int e = 127 - 32 + lz;
	rcp += uint32_t(e) << 23;
	return u2f(rcp);
}

static float RCP_FLOAT_LUT[256];
static bool rcp_float_lut_init = []() {
	for (int i = 0; i < 256; i++)
		RCP_FLOAT_LUT[i] = 1.0f / (1.0f + (float(i) + 0.5f) / 256.0f);
	return true;
}();

// rcp_float (gs/shaders/math_utils.h:65-101).
static float rcp_float(float v)
{
	uint32_t u = f2u(v);
	int e = int(bfe(u, 23, 8));
	if (e == 0)
		return u2f(0x7f800000u);
	int shifted = 127 - e;
	float x = RCP_FLOAT_LUT[bfe(u, 15, 8)];
	u &= (1u << 23) - 1u;
	u |= 127u << 23;
	float a = u2f(u);
	for (int it = 0; it < 4; it++)
	{
		float x2 = x * 2.0f;
		float xs = x * x;
		float xsa = xs * a;
		x = x2 - xsa;
	}
	return std::ldexp(x, shifted);
}

// ---------------------------------------------------------------------------
// Setup records (gs/shaders/data_structures.h:32-52).
struct Setup
{
	int32_t a[3], b[3], c[3];
	float inv_area, error_i, error_j;
	int32_t bb[4];
	uint32_t z[3];
};

struct TAttr
{
	float stqf0[4], stqf1[4], stqf2[4];
	uint32_t rgba0, rgba1, rgba2;
};

static bool tie_break(int32_t ex, int32_t ey) { return ey > 0 || (ey == 0 && ex < 0); }

static bool order_less(const int32_t a[2], const int32_t b[2], uint32_t az, uint32_t bz)
{
	if (bz != az) return az < bz;
	if (b[1] != a[1]) return a[1] < b[1];
	return a[0] < b[0];
}

static int32_t quantize_const(int64_t c) { return int32_t(uint32_t(uint64_t(c) >> 1)); }

struct Backend
{
	uint32_t rate_x = 0, rate_y = 0;
	uint32_t num_planes = 1;
	std::vector<uint8_t> vram;
	// Phase LUT of super-sampled texture filtering for the current rate.
	uint32_t phase_lut[64 * 64 * 2 + 32 * 32] = {};
	// Deinterlacer history: the last four merged fields, newest first.
	std::vector<uint32_t> fields[4];
	uint32_t field_w = 0, field_h = 0;
	std::vector<uint16_t> clut;
	uint32_t last_clut_instance = 0;
	std::vector<pgs_vertex_position> res_pos;
	std::vector<pgs_vertex_attribute> res_attr;
	std::vector<pgs_primitive_attribute> res_prim;
	std::atomic<uint64_t> fragments{0};
	// Primitive states after setup and the single-sample heuristic, appended
	// per render pass (for tests of the heuristic's decisions).
	std::vector<uint32_t> state_log;

	Backend() : clut(PGS_CLUT_INSTANCES * 512, 0)
	{
		vram.assign(VRAM, 0);
		res_pos.resize(3 * PGS_MAX_PRIMITIVES_PER_FLUSH);
		res_attr.resize(3 * PGS_MAX_PRIMITIVES_PER_FLUSH);
		res_prim.resize(PGS_MAX_PRIMITIVES_PER_FLUSH);
	}

	// Texels come from this copy of the VRAM planes, taken when a pass with
	// textures begins: textures are sampled as the pass found them (the
	// reference samples texture-cache images uploaded before the pass renders),
	// whatever the pass itself writes.
	std::vector<uint8_t> tex_vram;
	// Snapshots of every VRAM plane taken during the open pass
	// (snapshot_vram); textures the pass names decode from them instead.
	std::vector<uint8_t> snaps[PGS_MAX_VRAM_SNAPSHOTS];
	uint32_t snaps_taken = 0;
	static uint32_t t32(const uint8_t *src, uint32_t plane, uint32_t i) { return reinterpret_cast<const uint32_t *>(src + plane * size_t(VRAM))[i]; }
	static uint16_t t16(const uint8_t *src, uint32_t plane, uint32_t i) { return reinterpret_cast<const uint16_t *>(src + plane * size_t(VRAM))[i]; }
	static uint8_t t8(const uint8_t *src, uint32_t plane, uint32_t i) { return src[plane * size_t(VRAM) + i]; }
	uint32_t &w32(uint32_t plane, uint32_t i) { return reinterpret_cast<uint32_t *>(vram.data() + plane * size_t(VRAM))[i]; }
	uint16_t &w16(uint32_t plane, uint32_t i) { return reinterpret_cast<uint16_t *>(vram.data() + plane * size_t(VRAM))[i]; }
	uint8_t &w8(uint32_t plane, uint32_t i) { return vram[plane * size_t(VRAM) + i]; }

	// -----------------------------------------------------------------------
	// triangle_setup.comp main_inner.
	void triangle_setup(uint32_t index, const pgs_vertex_position *vp, const pgs_vertex_attribute *va,
	                    pgs_primitive_attribute &pa, Setup &out, TAttr &ta, const uint32_t *opaque_fbmasks,
	                    int srx, int sry, uint32_t packed_z_shift, int32_t &bucket_out,
	                    const pgs_render_pass *rp = nullptr, uint32_t blur_mask = 0, bool force_linear = false)
	{
		bucket_out = -1;
		int order[3] = { 0, 1, 2 };
		uint32_t st = pa.state;
		bool parallelogram = bfe(st, 15, 1);
		bool perspective = bfe(st, 18, 1);
		bool iip = bfe(st, 19, 1);
		bool fix = bfe(st, 20, 1);
		bool sprite = bfe(st, 21, 1);
		bool line = bfe(st, 22, 1);
		bool multisample = bfe(st, 16, 1);
		uint32_t provoking = bfe(st, 27, 2);
		uint32_t instance = bfe(st, 29, 3);
		uint32_t opaque_fbmask = opaque_fbmasks[instance];

		int32_t a[2] = { vp[3 * index].x, vp[3 * index].y };
		int32_t b[2] = { vp[3 * index + 1].x, vp[3 * index + 1].y };
		int32_t c[2] = { vp[3 * index + 2].x, vp[3 * index + 2].y };
		uint32_t za = vp[3 * index].z, zb = vp[3 * index + 1].z, zc = vp[3 * index + 2].z;

		if (line)
		{
			bool sax = (a[0] & 15) == 0, say = (a[1] & 15) == 0;
			bool sbx = (b[0] & 15) == 0, sby = (b[1] & 15) == 0;
			if ((sax || sbx) && b[0] > a[0]) { a[0] += 1; b[0] += 1; }
			if ((say || sby) && b[1] > a[1]) { a[1] += 1; b[1] += 1; }
		}

		if ((!parallelogram || line) && !fix)
		{
			if (!line && !order_less(b, c, zb, zc))
			{
				std::swap(order[1], order[2]);
				std::swap(b[0], c[0]); std::swap(b[1], c[1]);
				std::swap(zb, zc);
			}
			if (!order_less(a, b, za, zb))
			{
				std::swap(order[0], order[1]);
				std::swap(a[0], b[0]); std::swap(a[1], b[1]);
				std::swap(za, zb);
			}
		}
		else if (provoking == 1)
		{
			std::swap(order[0], order[1]);
			std::swap(a[0], b[0]); std::swap(a[1], b[1]);
			std::swap(za, zb);
		}
		else if (provoking == 2)
		{
			std::swap(order[0], order[2]);
			std::swap(a[0], c[0]); std::swap(a[1], c[1]);
			std::swap(za, zc);
		}

		if (sprite)
		{
			c[0] = a[0]; c[1] = b[1];
			b[1] = a[1];
		}
		else if (line)
		{
			int32_t abx = b[0] - a[0], aby = b[1] - a[1];
			if (std::abs(abx) >= std::abs(aby))
			{
				int32_t sgn = (abx > 0) - (abx < 0);
				int32_t yd = -sgn * 8;
				if (multisample) yd *= 2;
				c[1] = a[1] + yd;
				a[1] -= yd;
				b[1] -= yd;
				if (!multisample) { a[1] += 1; b[1] += 1; }
				c[0] = a[0];
			}
			else
			{
				int32_t sgn = (aby > 0) - (aby < 0);
				int32_t xd = sgn * 8;
				if (multisample) xd *= 2;
				c[0] = a[0] + xd;
				a[0] -= xd;
				b[0] -= xd;
				if (!multisample) { a[0] += 1; b[0] += 1; }
				c[1] = a[1];
			}
		}

		int32_t ab[2] = { b[0] - a[0], b[1] - a[1] };
		int32_t ac[2] = { c[0] - a[0], c[1] - a[1] };
		int64_t signed_area = int64_t(ab[1]) * ac[0] - int64_t(ab[0]) * ac[1];

		if (signed_area == 0)
		{
			out.bb[0] = 0; out.bb[1] = 0; out.bb[2] = -1; out.bb[3] = -1;
			if (sry != 0)
				pa.state |= 1u << 26;
			return;
		}

		uint32_t area;
		bool flipped = signed_area < 0;
		if (flipped)
		{
			area = uint32_t(-uint64_t(signed_area));
			std::swap(ab[0], ac[0]); std::swap(ab[1], ac[1]);
			std::swap(b[0], c[0]); std::swap(b[1], c[1]);
			std::swap(zb, zc);
			std::swap(order[1], order[2]);
		}
		else
			area = uint32_t(uint64_t(signed_area));

		int32_t bc[2] = { c[0] - b[0], c[1] - b[1] };
		int32_t ca[2] = { -ac[0], -ac[1] };

		int32_t dcdx = ab[1], dcdy = -ab[0];
		int32_t dadx = bc[1], dady = -bc[0];
		int32_t dbdx = ca[1], dbdy = -ca[0];

		int64_t const_c = int64_t(-a[0]) * dcdx - int64_t(a[1]) * dcdy;
		int64_t const_a = int64_t(-b[0]) * dadx - int64_t(b[1]) * dady;
		int64_t const_b = int64_t(-c[0]) * dbdx - int64_t(c[1]) * dbdy;

		bool tba = tie_break(bc[0], bc[1]);
		bool tbb = tie_break(ca[0], ca[1]);
		bool tbc = tie_break(ab[0], ab[1]);
		int32_t err_a = !tba, err_b = !tbb, err_c = !tbc;
		const_a -= err_a;
		const_b -= err_b;
		const_c -= err_c;
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
		float inv_area_scaled = inv_area * 2.0f;
		float error_i = float(err_b) * inv_area;
		float error_j = float(err_c) * inv_area;

		if (sprite) { zb = za; zc = za; }
		else if (line) { zc = za; }

		if (fix || sprite) { order[0] = 0; order[1] = 1; order[2] = 2; }

		const pgs_vertex_attribute &at0 = va[3 * index + order[0]];
		const pgs_vertex_attribute &at1 = va[3 * index + order[1]];
		pgs_vertex_attribute at2 = {};
		if (!sprite && !line)
			at2 = va[3 * index + order[2]];

		float s0[4], s1[4], s2[4] = { 0, 0, 0, 0 };
		if (perspective)
		{
			s0[0] = at0.s; s0[1] = at0.t; s0[2] = at0.q; s0[3] = at0.fog;
			s1[0] = at1.s; s1[1] = at1.t; s1[2] = at1.q; s1[3] = at1.fog;
			if (!sprite && !line) { s2[0] = at2.s; s2[1] = at2.t; s2[2] = at2.q; s2[3] = at2.fog; }
		}
		else
		{
			s0[0] = float(at0.u) / 16.0f; s0[1] = float(at0.v) / 16.0f; s0[2] = at0.q; s0[3] = at0.fog;
			s1[0] = float(at1.u) / 16.0f; s1[1] = float(at1.v) / 16.0f; s1[2] = at1.q; s1[3] = at1.fog;
			if (!sprite && !line)
			{
				s2[0] = float(at2.u) / 16.0f; s2[1] = float(at2.v) / 16.0f; s2[2] = at2.q; s2[3] = at2.fog;
			}
		}

		if (sprite)
		{
			float o0[4] = { s0[0], s0[1], s0[2], s0[3] }, o1[4] = { s1[0], s1[1], s1[2], s1[3] };
			if (flipped)
			{
				s2[0] = o1[0]; s2[1] = o0[1]; s2[2] = o0[2]; s2[3] = o0[3];
				s1[0] = o0[0]; s1[1] = o1[1]; s1[2] = o0[2]; s1[3] = o0[3];
			}
			else
			{
				s2[0] = o0[0]; s2[1] = o1[1]; s2[2] = o0[2]; s2[3] = o0[3];
				s1[0] = o1[0]; s1[1] = o0[1]; s1[2] = o0[2]; s1[3] = o0[3];
			}
		}
		else if (line)
		{
			memcpy(s2, s0, sizeof(s2));
		}

		if (perspective)
		{
			if (s0[2] < 0.0f)
			{
				s0[0] = -s0[0]; s0[1] = -s0[1];
				s1[0] = -s1[0]; s1[1] = -s1[1];
				s2[0] = -s2[0]; s2[1] = -s2[1];
			}
			s0[2] = std::fabs(s0[2]); s1[2] = std::fabs(s1[2]); s2[2] = std::fabs(s2[2]);
			uint32_t qexp = bfe(f2u(std::max(std::max(s0[2], s1[2]), s2[2])), 23, 8);
			s0[2] = u2f(f2u(s0[2]) & ~0xffu);
			s1[2] = u2f(f2u(s1[2]) & ~0xffu);
			s2[2] = u2f(f2u(s2[2]) & ~0xffu);
			uint32_t sexp = bfe(f2u(std::max(std::max(std::fabs(s0[0]), std::fabs(s1[0])), std::fabs(s2[0]))), 23, 8);
			uint32_t texp = bfe(f2u(std::max(std::max(std::fabs(s0[1]), std::fabs(s1[1])), std::fabs(s2[1]))), 23, 8);
			uint32_t schop = std::min<uint32_t>(9 + std::max(sexp, qexp) - sexp, 23);
			uint32_t tchop = std::min<uint32_t>(9 + std::max(texp, qexp) - texp, 23);
			uint32_t smask = ~((1u << schop) - 1u), tmask = ~((1u << tchop) - 1u);
			s0[0] = u2f(f2u(s0[0]) & smask); s1[0] = u2f(f2u(s1[0]) & smask); s2[0] = u2f(f2u(s2[0]) & smask);
			s0[1] = u2f(f2u(s0[1]) & tmask); s1[1] = u2f(f2u(s1[1]) & tmask); s2[1] = u2f(f2u(s2[1]) & tmask);

			bool needs_lod = (pa.tex2 & 1u) == 0;
			if (!needs_lod && s0[2] == s1[2] && s0[2] == s2[2])
			{
				float inv_q = rcp_float(s0[2]);
				s0[0] *= inv_q; s0[1] *= inv_q;
				s1[0] *= inv_q; s1[1] *= inv_q;
				s2[0] *= inv_q; s2[1] *= inv_q;
				s0[2] = 1.0f; s1[2] = 1.0f; s2[2] = 1.0f;
			}
		}

		float di[4], dj[4];
		for (int k = 0; k < 4; k++)
		{
			di[k] = fix ? 0.0f : (s1[k] - s0[k]);
			dj[k] = fix ? 0.0f : (s2[k] - s0[k]);
		}
		memcpy(ta.stqf0, s0, sizeof(s0));
		memcpy(ta.stqf1, di, sizeof(di));
		memcpy(ta.stqf2, dj, sizeof(dj));

		if (iip && !sprite)
		{
			uint32_t r0 = at0.rgba, r1 = at1.rgba, r2 = at2.rgba;
			if (fix) r1 = r0;
			if (fix || line) r2 = r0;
			ta.rgba0 = r0; ta.rgba1 = r1; ta.rgba2 = r2;
		}
		else
		{
			uint32_t flat = va[3 * index].rgba;
			ta.rgba0 = ta.rgba1 = ta.rgba2 = flat;
		}

		int32_t pa_[3] = { dadx, dady, quantize_const(const_a) };
		int32_t pb_[3] = { dbdx, dbdy, quantize_const(const_b) };
		int32_t pc_[3] = { dcdx, dcdy, quantize_const(const_c) };
		uint32_t ax = uint32_t(pa_[0]) << 6;
		ax = (ax & ~1u) | uint32_t(parallelogram);
		ax = (ax & ~(3u << 2)) | ((uint32_t(flip_b) & 3u) << 2);
		ax = (ax & ~(3u << 4)) | ((uint32_t(flip_c) & 3u) << 4);
		pa_[0] = int32_t(ax);

		int32_t d[2];
		if (parallelogram) { d[0] = b[0] + c[0] - a[0]; d[1] = b[1] + c[1] - a[1]; }
		else { d[0] = c[0]; d[1] = c[1]; }

		int32_t di_r = 0, dj_r = 0;
		if (sprite)
		{
			int32_t xd = d[0] - a[0], yd = d[1] - a[1];
			bool right = xd > 0 && (xd & (xd - 1)) != 0;
			bool bottom = yd > 0 && (yd & (yd - 1)) != 0;
			if (right) { di_r += pb_[0]; dj_r += pc_[0]; }
			if (bottom) { di_r += pb_[1]; dj_r += pc_[1]; }
		}
		else if (parallelogram && !perspective)
		{
			bool nearest = (pa.tex & (1u << 16)) == 0;
			bool npot_area = (area & (area - 1)) != 0;
			if (nearest && npot_area)
			{
				int32_t d0x = int32_t(at0.u) - a[0], d0y = int32_t(at0.v) - a[1];
				int32_t d1x = int32_t(at1.u) - b[0], d1y = int32_t(at1.v) - b[1];
				int32_t d2x = int32_t(at2.u) - c[0], d2y = int32_t(at2.v) - c[1];
				if (d0x == d1x && d0y == d1y && d0x == d2x && d0y == d2y)
				{
					bool mis_x = (std::min(a[0], d[0]) & 15) != 0;
					bool mis_y = (std::min(a[1], d[1]) & 15) != 0;
					float dudx = di[0] * float(pb_[0]) + dj[0] * float(pc_[0]);
					float dvdx = di[1] * float(pb_[0]) + dj[1] * float(pc_[0]);
					float dudy = di[0] * float(pb_[1]) + dj[0] * float(pc_[1]);
					float dvdy = di[1] * float(pb_[1]) + dj[1] * float(pc_[1]);
					bool adj_x = mis_x && ((dudx > 0.0f && dvdx == 0.0f) || (dvdx > 0.0f && dudx == 0.0f));
					bool adj_y = mis_y && ((dudy > 0.0f && dvdy == 0.0f) || (dvdy > 0.0f && dudy == 0.0f));
					if (adj_x) { di_r -= pb_[0]; dj_r -= pc_[0]; }
					if (adj_y) { di_r -= pb_[1]; dj_r -= pc_[1]; }
				}
			}
		}

		float eighth = 0.125f * inv_area_scaled;
		float ti = float(di_r) * eighth;
		float tj = float(dj_r) * eighth;
		error_i = error_i + ti;
		error_j = error_j + tj;

		memcpy(out.a, pa_, sizeof(pa_));
		memcpy(out.b, pb_, sizeof(pb_));
		memcpy(out.c, pc_, sizeof(pc_));
		out.inv_area = inv_area_scaled;
		out.error_i = error_i;
		out.error_j = error_j;
		out.z[0] = za;
		out.z[1] = f2u(float(uint32_t(zb - za)));
		out.z[2] = f2u(float(uint32_t(zc - za)));

		// pack_bounding_box (gs/shaders/intersect.h:83-104) and clip.
		int32_t lo[2] = { std::min(std::min(a[0], b[0]), std::min(c[0], d[0])),
		                  std::min(std::min(a[1], b[1]), std::min(c[1], d[1])) };
		int32_t hi[2] = { std::max(std::max(a[0], b[0]), std::max(c[0], d[0])),
		                  std::max(std::max(a[1], b[1]), std::max(c[1], d[1])) };
		lo[0] = (lo[0] + (15 >> sry)) >> 4;
		lo[1] = (lo[1] + (15 >> sry)) >> 4;
		hi[0] = (hi[0] - 1) >> 4;
		hi[1] = (hi[1] - 1) >> 4;
		if (multisample && !line)
		{
			lo[0] -= 1; lo[1] -= 1;
			hi[0] += 1; hi[1] += 1;
		}
		out.bb[0] = std::max(lo[0], int32_t(pa.bb[0]));
		out.bb[1] = std::max(lo[1], int32_t(pa.bb[1]));
		out.bb[2] = std::min(hi[0], int32_t(pa.bb[2]));
		out.bb[3] = std::min(hi[1], int32_t(pa.bb[3]));

		if (sprite && !perspective)
		{
			int32_t u0x = int32_t(at0.u) - a[0], u0y = int32_t(at0.v) - a[1];
			int32_t u1x = int32_t(at1.u) - d[0], u1y = int32_t(at1.v) - d[1];
			int32_t mnx = std::min(u0x, u1x), mny = std::min(u0y, u1y);
			int32_t mxx = std::max(u0x, u1x), mxy = std::max(u0y, u1y);
			bool csx = (mnx & 15) == 8, csy = (mny & 15) == 8;
			bool nsx = (mxx & 15) == 9, nsy = (mxy & 15) == 9;
			int32_t dx = std::abs(d[0] - a[0]), dy = std::abs(d[1] - a[1]);
			nsx = nsx && (dx & (dx - 1)) != 0;
			nsy = nsy && (dy & (dy - 1)) != 0;
			bool no_interp = (mxx - mnx) <= 1 && (mxy - mny) <= 1;
			bool half = (nsx || csx) && (nsy || csy);
			if (half && no_interp)
				pa.tex &= ~(1u << 16);
		}

		uint32_t s = pa.state;
		if (pa.fbmsk != opaque_fbmask && (s & (1u << 14)) != 0)
			pa.state = s & ~(1u << 14);

		// Super-sampled textures (triangle_setup.comp:677-825): per sprite,
		// sample-to-sample mapping for nearest blits and perspective, the
		// single-sampled layer for nearest downsamples and blur kernels, the
		// resolved layer for linear upsamples (force_linear, for field
		// rendering: blur kernels read the resolved layer linearly, linear
		// downsamples and upsamples stay per sample); per-sample interpolation
		// (no attribute snap, i/j moved to the mean sample position) for what
		// stays per-sample.
		const uint32_t PER_SAMPLE = 1u << 24, MAPPING = 1u << 25, RESOLVED = 1u << 26;
		if (sry != 0 && rp && (pa.tex & (PER_SAMPLE | MAPPING)) == PER_SAMPLE)
		{
			uint32_t tex = pa.tex;
			const int32_t udx = std::abs(int32_t(at1.u) - int32_t(at0.u)), udy = std::abs(int32_t(at1.v) - int32_t(at0.v));
			const int32_t ddx = std::abs(d[0] - a[0]), ddy = std::abs(d[1] - a[1]);
			if ((tex & (1u << 16)) == 0)
			{
				if (perspective)
					tex |= MAPPING;
				else if (udx > ddx + 1 || udy > ddy + 1)
					tex &= ~PER_SAMPLE;
				else if (udx >= ddx - 16 || udy >= ddy - 16)
				{
					const uint32_t bm = rp->states[std::min<uint32_t>(pa.state & 0xfffu, std::max<uint32_t>(rp->num_states, 1) - 1)].blend_mode;
					const uint32_t inst = bfe(pa.state, 29, 3);
					const bool blur = ((blur_mask >> inst) & 1u) && (bm & (1u << 9)) && !(pa.state & (1u << 12)) &&
					                  bfe(bm, 11, 2) == 0 && bfe(bm, 13, 2) == 2 && bfe(bm, 17, 2) == 1;
					if (blur && force_linear)
					{
						// Field rendering keeps blur kernels per sample: the
						// resolved layer, filtered linearly, with the mean
						// sample position moved to the texel centre
						// (triangle_setup.comp:729-746).
						tex |= RESOLVED | (1u << 16);
						const int32_t avg_u = (int32_t(at0.u) + int32_t(at1.u)) >> 1;
						const int32_t avg_v = (int32_t(at0.v) + int32_t(at1.v)) >> 1;
						const int32_t avg_x = (d[0] + a[0]) >> 1, avg_y = (d[1] + a[1]) >> 1;
						const int32_t ph_x = (avg_u - avg_x) & 15, ph_y = (avg_v - avg_y) & 15;
						ta.stqf0[0] = ta.stqf0[0] + (0.5f - float(ph_x) / 16.0f);
						ta.stqf0[1] = ta.stqf0[1] + (0.5f - float(ph_y) / 16.0f);
					}
					else if (blur)
						tex &= ~PER_SAMPLE;
					else
						tex |= MAPPING;
				}
			}
			else if (!perspective)
			{
				if (udx > ddx + 1 && udy > ddy + 1)
				{
					if (!force_linear)
						tex &= ~PER_SAMPLE;
				}
				else if (ddx >= 2 * udx && ddy >= 2 * udy)
				{
					if (!force_linear)
						tex |= RESOLVED;
				}
			}
			pa.tex = tex;
			if ((tex & (PER_SAMPLE | MAPPING)) == PER_SAMPLE)
			{
				pa.state &= ~(1u << 26);
				const float corner = 8.0f * average_sampling_offset(uint32_t(srx), uint32_t(sry));
				const float di_dcorner = float(pb_[0] + pb_[1]) * corner;
				const float dj_dcorner = float(pc_[0] + pc_[1]) * corner;
				out.error_i = out.error_i - di_dcorner * inv_area_scaled;
				out.error_j = out.error_j - dj_dcorner * inv_area_scaled;
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
				// triangle_setup.comp:836-871: flat primitive, register the
				// depth bucket (Z >> z_shift_to_bucket * 8, clamped to 255).
				if (!line)
					pa.state |= 1u << 26;
				uint32_t z_shift = bfe(packed_z_shift, 4 * instance, 4) * 8;
				bucket_out = int32_t(std::min<uint32_t>(255u, za >> z_shift));
			}
		}
	}

	// -----------------------------------------------------------------------
	// triangle_setup_intersects_tile (gs/shaders/intersect.h:24-81).
	static bool intersects_tile(const Setup &s, int32_t lo0, int32_t lo1, int32_t hi0, int32_t hi1, bool ms_tri)
	{
		int32_t lo[2] = { std::max(s.bb[0], lo0), std::max(s.bb[1], lo1) };
		int32_t hi[2] = { std::min(s.bb[2], hi0), std::min(s.bb[3], hi1) };
		if (!(hi[0] >= lo[0] && hi[1] >= lo[1]))
			return false;
		int32_t ax = s.a[0];
		bool par = (ax & 1) != 0;
		int32_t off_b = int32_t(bfe(uint32_t(ax), 2, 2)) - 1;
		int32_t off_c = int32_t(bfe(uint32_t(ax), 4, 2)) - 1;
		ax >>= 6;
		int32_t A[3] = { ax, s.a[1], s.a[2] };
		lo[0] <<= 3; lo[1] <<= 3;
		hi[0] = (hi[0] << 3) | 7; hi[1] = (hi[1] << 3) | 7;
		auto dot = [](const int32_t *p, int32_t x, int32_t y) { return int32_t(uint32_t(p[0]) * uint32_t(x) + uint32_t(p[1]) * uint32_t(y) + uint32_t(p[2])); };
		auto pick = [&](int32_t v, int k) { return v >= 0 ? hi[k] : lo[k]; };
		int32_t da = dot(A, pick(A[0], 0), pick(A[1], 1));
		int32_t db = dot(s.b, pick(s.b[0], 0), pick(s.b[1], 1));
		int32_t dc = dot(s.c, pick(s.c[0], 0), pick(s.c[1], 1));
		if (ms_tri && !par)
		{
			da += 8 * std::max(std::abs(A[0]), std::abs(A[1]));
			db += 8 * std::max(std::abs(s.b[0]), std::abs(s.b[1]));
			dc += 8 * std::max(std::abs(s.c[0]), std::abs(s.c[1]));
		}
		bool ok = da >= 0 && db >= 0 && dc >= 0;
		if (par && !ok)
		{
			int32_t oa0 = pick(A[0], 0), oa1 = pick(A[1], 1);
			int32_t ob0 = (-s.c[0] >= 0) ? hi[0] : lo[0], ob1 = (-s.c[1] >= 0) ? hi[1] : lo[1];
			int32_t oc0 = (-s.b[0] >= 0) ? hi[0] : lo[0], oc1 = (-s.b[1] >= 0) ? hi[1] : lo[1];
			da = dot(A, oa0, oa1);
			db = dot(s.b, ob0, ob1);
			dc = dot(s.c, oc0, oc1);
			db += da + off_b;
			dc += da + off_c;
			int32_t fa0 = A[0] >= 0 ? lo[0] : hi[0], fa1 = A[1] >= 0 ? lo[1] : hi[1];
			da = dot(A, fa0, fa1);
			ok = (-1 >= da) && db >= 0 && dc >= 0;
		}
		return ok;
	}

	// -----------------------------------------------------------------------
	// Per pass state.
	struct PassCtx
	{
		const pgs_render_pass *rp;
		const uint8_t *const *tex_src; // VRAM each texture decodes from
		const pgs_primitive_attribute *prims;
		const Setup *setup;
		const TAttr *tattr;
		uint32_t sr_dim_log2, num_samples, sr_x_log2;
		bool ss;                 // this work item is super-sampled
		bool has_ss_reference;   // VRAM holds sample planes
		uint32_t fb_psm, zb_psm; // effective formats; zb_psm = ~0u when not Z sensitive
		uint32_t fb_base, fb_stride, zb_base;
		int32_t snap_mask_x, snap_mask_y; // raster snap; y halves when field rendering
		bool preserve_samples;
		bool has_aa1, has_scanmsk;
		bool tex_array;          // some texture of the pass is super-sampled
		const uint8_t *zcache;   // depth read from this VRAM snapshot when set
	};

	struct Request
	{
		int coverage = 0;
		bool z_test = false, z_write = false, multisample = false, perspective = false, z_greater = false;
		uint32_t z = 0, state = 0;
		float i = 0, j = 0;
	};

	struct Sample
	{
		uint32_t color, depth;
		bool color_dirty, depth_dirty;
		int32_t hx, hy; // high-resolution coordinate
		Request pending;
		uint32_t pending_prim;
		uint32_t index; // sample index within the pixel
	};

	// evaluate_coverage (gs/shaders/intersect.h:156-244).
	static int evaluate_coverage(const Setup &s, int32_t cx, int32_t cy, float &i, float &j, bool ms, bool line, int dim)
	{
		int32_t sx = cx >> dim, sy = cy >> dim;
		if (!(sx >= s.bb[0] && sy >= s.bb[1] && s.bb[2] >= sx && s.bb[3] >= sy))
			return 0;
		int32_t ax = s.a[0];
		bool par = (ax & 1) != 0;
		int32_t off_b = int32_t(bfe(uint32_t(ax), 2, 2)) - 1;
		int32_t off_c = int32_t(bfe(uint32_t(ax), 4, 2)) - 1;
		ax >>= 6;
		int32_t px = cx << (3 - dim), py = cy << (3 - dim);
		auto dot3 = [](int32_t p0, int32_t p1, int32_t p2, int32_t x, int32_t y) {
			return int32_t(uint32_t(p0) * uint32_t(x) + uint32_t(p1) * uint32_t(y) + uint32_t(p2));
		};
		int32_t ea = dot3(ax, s.a[1], s.a[2], px, py);
		int32_t eb = dot3(s.b[0], s.b[1], s.b[2], px, py);
		int32_t ec = dot3(s.c[0], s.c[1], s.c[2], px, py);
		float ir = float(eb) * s.inv_area;
		ir = ir + s.error_i;
		float jr = float(ec) * s.inv_area;
		jr = jr + s.error_j;
		i = ir;
		j = jr;
		if (par && ea < 0)
		{
			eb += ea + off_b;
			ec += ea + off_c;
			ea = 0;
		}
		bool center = ea >= 0 && eb >= 0 && ec >= 0;
		int count = 0;
		if (ms && line)
		{
			if (center)
				count = int(std::max(0.0f, 128.0f - 256.0f * std::fabs(0.5f - j)));
		}
		else if (center)
			count = 0x80;
		else if (ms && !par)
		{
			bool ba = dot3(ax, s.a[1], s.a[2], px, py) >= 0;
			bool bb = dot3(s.b[0], s.b[1], s.b[2], px, py) >= 0;
			bool bc = dot3(s.c[0], s.c[1], s.c[2], px, py) >= 0;
			if (int(ba) + int(bb) + int(bc) == 2)
			{
				float neg;
				int32_t md;
				if (!ba)
				{
					md = std::max(std::abs(s.b[0] + s.c[0]), std::abs(s.b[1] + s.c[1]));
					neg = (i + j) - 1.0f;
				}
				else if (!bb)
				{
					md = std::max(std::abs(s.b[0]), std::abs(s.b[1]));
					neg = -i;
				}
				else
				{
					md = std::max(std::abs(s.c[0]), std::abs(s.c[1]));
					neg = -j;
				}
				float scaled = float(md) * s.inv_area;
				float until = neg / scaled;
				float fc = 8.0f - until;
				count = int(std::min(std::max(16.0f * fc, 0.0f), 127.0f));
			}
		}
		return count;
	}

	static void barycentric(const Setup &s, int32_t cx, int32_t cy, int dim, float &i, float &j)
	{
		int32_t px = cx << (3 - dim), py = cy << (3 - dim);
		int32_t eb = int32_t(uint32_t(s.b[0]) * uint32_t(px) + uint32_t(s.b[1]) * uint32_t(py) + uint32_t(s.b[2]));
		int32_t ec = int32_t(uint32_t(s.c[0]) * uint32_t(px) + uint32_t(s.c[1]) * uint32_t(py) + uint32_t(s.c[2]));
		float ir = float(eb) * s.inv_area;
		i = ir + s.error_i;
		float jr = float(ec) * s.inv_area;
		j = jr + s.error_j;
	}

	// shade_early (gs/shaders/ubershader.comp:782-910).
	Request shade_early(const PassCtx &P, uint32_t pi, const Sample &smp, bool &opaque)
	{
		const Setup &s = P.setup[pi];
		uint32_t st = P.prims[pi].state;
		Request r;
		opaque = bfe(st, 14, 1);
		bool zs = P.zb_psm != ~0u;
		if (zs)
		{
			r.z_test = bfe(st, 12, 1);
			r.z_write = bfe(st, 13, 1);
			r.z_greater = bfe(st, 17, 1);
		}
		r.state = st & 0xfffu;
		r.multisample = P.has_aa1 && bfe(st, 16, 1);
		r.perspective = bfe(st, 18, 1);
		int dim = int(P.sr_dim_log2);
		int32_t rx = smp.hx, ry = smp.hy;
		if (P.ss && (st & (1u << 25)))
		{
			// Sample-mapped textures keep the full-rate row grid when the
			// rows are snapped for field rendering (ubershader.comp:816-821).
			rx &= P.snap_mask_x;
			ry &= (P.tex_array && (P.prims[pi].tex & (1u << 25))) ? P.snap_mask_x : P.snap_mask_y;
		}
		float i = 0, j = 0;
		r.coverage = evaluate_coverage(s, rx, ry, i, j, r.multisample, bfe(st, 22, 1), dim);

		if (P.has_scanmsk)
		{
			int32_t sy = smp.hy;
			if (st & (1u << 21))
				sy >>= dim;
			if ((sy & 1) == 0) { if (bfe(st, 23, 1)) r.coverage = 0; }
			else if (bfe(st, 24, 1)) r.coverage = 0;
		}

		if (zs && r.multisample && r.coverage < 0x80)
			r.z_write = false;

		uint32_t z = s.z[0];
		float dzdi = u2f(s.z[1]), dzdj = u2f(s.z[2]);
		float t0 = dzdi * i;
		float t1 = dzdj * j;
		float zf = round_even(t0 + t1);
		zf = std::min(std::max(zf, 0.0f), 4294967040.0f);
		uint32_t dz = uint32_t(zf);
		dz = std::min(dz, 0xffffffffu - z);
		z += dz;
		if (zs && is16(P.zb_psm)) z = std::min(z, 0xffffu);
		else if (zs && is24(P.zb_psm)) z = std::min(z, 0xffffffu);

		if (P.ss && r.coverage != 0)
		{
			uint32_t snap = st & ((1u << 25) | (1u << 26));
			if (snap == (1u << 26))
				barycentric(s, smp.hx & P.snap_mask_x, smp.hy & P.snap_mask_y, dim, i, j);
			else if (P.tex_array && snap == (1u << 25))
				// Per-sample textured sprite: coverage snapped, attributes
				// interpolated per sample (ubershader.comp:888-895).
				barycentric(s, smp.hx, smp.hy, dim, i, j);
		}
		r.z = z;
		r.i = i;
		r.j = j;
		return r;
	}

	// Texel fetch from VRAM + CLUT (upload.comp decode).
	uint32_t clut_color(const pgs_texture_desc &t, uint32_t index)
	{
		uint32_t bi = t.csa * 16 + index;
		bool c16 = t.cpsm == CT16 || t.cpsm == CT16S;
		if (t.psm == T8 || t.psm == T8H)
		{
			uint32_t bank = std::min<uint32_t>(bi >> 4, c16 ? 31u : 15u);
			bi = bank * 16 + (bi & 15);
		}
		const uint16_t *cl = &clut[size_t(t.clut_instance) * 512];
		if (c16)
		{
			uint32_t c = cl[bi];
			uint32_t r = (c & 0x1f) << 3, g = ((c >> 5) & 0x1f) << 3, b = ((c >> 10) & 0x1f) << 3;
			uint32_t a = (t.aem && c == 0) ? 0 : ((c & 0x8000) ? t.ta1 : t.ta0);
			return r | (g << 8) | (b << 16) | (a << 24);
		}
		return uint32_t(cl[bi]) | (uint32_t(cl[bi + 256]) << 16);
	}

	uint32_t texel(const uint8_t *src, const pgs_texture_desc &t, uint32_t level, int32_t x, int32_t y)
	{
		uint32_t tbp = level ? (t.mip[level - 1] & 0x3fffu) : t.tbp0;
		uint32_t tbw = level ? (t.mip[level - 1] >> 16) : t.tbw;
		uint32_t a = swizzle(uint32_t(x), uint32_t(y), tbp, tbw, t.psm);
		switch (t.psm)
		{
		case CT24: case Z24:
		{
			uint32_t c = t32(src, 0, a) & 0xffffffu;
			uint32_t al = (t.aem && c == 0) ? 0 : t.ta0;
			return c | (al << 24);
		}
		case CT16: case CT16S: case Z16: case Z16S:
		{
			uint32_t c = t16(src, 0, a);
			uint32_t r = (c & 0x1f) << 3, g = ((c >> 5) & 0x1f) << 3, b = ((c >> 10) & 0x1f) << 3;
			uint32_t al = (t.aem && c == 0) ? 0 : ((c & 0x8000) ? t.ta1 : t.ta0);
			return r | (g << 8) | (b << 16) | (al << 24);
		}
		case T8: return clut_color(t, t8(src, 0, a));
		case T8H: return clut_color(t, t32(src, 0, a) >> 24);
		case T4:
		{
			uint32_t byte = t8(src, 0, a >> 1);
			return clut_color(t, (byte >> ((a & 1) * 4)) & 15u);
		}
		case T4HL: return clut_color(t, (t32(src, 0, a) >> 24) & 15u);
		case T4HH: return clut_color(t, t32(src, 0, a) >> 28);
		default: return t32(src, 0, a);
		}
	}

	static int32_t wrap_coord(int32_t v, uint32_t mode, uint32_t size_log2, uint32_t lo, uint32_t hi)
	{
		int32_t size = 1 << size_log2;
		switch (mode)
		{
		case 0: return v & (size - 1);
		case 1: return std::min(std::max(v, 0), size - 1);
		case 2: return std::min(std::max(v, int32_t(lo)), int32_t(hi));
		default: return int32_t(((uint32_t(v) & uint32_t(size - 1)) & lo) | hi);
		}
	}

	// One filtered sample of mip level `level`: coordinates as sample_texture
	// (gs/shaders/ubershader.comp:1133-1151,1214-1227), region bounds and masks
	// shifted down by the level (texture_clamp :947-953; upload_texture
	// gs/gs_renderer.cpp:3578-3590), bilinear as exact k/16 weights + roundEven.
	void sample_level(const uint8_t *src, const pgs_texture_desc &t, uint32_t level, bool clamp_s, bool clamp_t, bool linear, float u,
	                  float v, bool perspective, uint32_t rgba[4])
	{
		uint32_t twl = t.tw_log2 - level, thl = t.th_log2 - level;
		float uu, vv;
		if (perspective)
		{
			uu = u * float(1u << twl);
			vv = v * float(1u << thl);
		}
		else
		{
			float scale = std::ldexp(1.0f, -int(level));
			uu = u * scale;
			vv = v * scale;
		}
		uint32_t minu = t.minu >> level, maxu = t.maxu >> level, minv = t.minv >> level, maxv = t.maxv >> level;
		if (clamp_s)
		{
			float lo = (t.wms == 2) ? float(minu) : 0.0f;
			float hi = (t.wms == 2) ? float(maxu) : float((1u << twl) - 1u);
			uu = std::min(std::max(uu, lo + 0.5f), hi + 0.5f);
		}
		if (clamp_t)
		{
			float lo = (t.wmt == 2) ? float(minv) : 0.0f;
			float hi = (t.wmt == 2) ? float(maxv) : float((1u << thl) - 1u);
			vv = std::min(std::max(vv, lo + 0.5f), hi + 0.5f);
		}
		float fu = uu * 16.0f;
		fu = fu + (1.0f / 64.0f);
		float fv = vv * 16.0f;
		fv = fv + (1.0f / 64.0f);
		int32_t ku = int32_t(std::floor(fu));
		int32_t kv = int32_t(std::floor(fv));
		if (!linear)
		{
			int32_t x = wrap_coord(ku >> 4, t.wms, twl, minu, maxu);
			int32_t y = wrap_coord(kv >> 4, t.wmt, thl, minv, maxv);
			uint32_t c = texel(src, t, level, x, y);
			for (int k = 0; k < 4; k++)
				rgba[k] = (c >> (8 * k)) & 0xffu;
			return;
		}
		int32_t bu = ku - 8, bv = kv - 8;
		int32_t x0 = bu >> 4, y0 = bv >> 4;
		uint32_t fx = uint32_t(bu) & 15u, fy = uint32_t(bv) & 15u;
		int32_t xs[2] = { wrap_coord(x0, t.wms, twl, minu, maxu), wrap_coord(x0 + 1, t.wms, twl, minu, maxu) };
		int32_t ys[2] = { wrap_coord(y0, t.wmt, thl, minv, maxv), wrap_coord(y0 + 1, t.wmt, thl, minv, maxv) };
		uint32_t wx[2] = { 16 - fx, fx }, wy[2] = { 16 - fy, fy };
		uint32_t acc[4] = { 0, 0, 0, 0 };
		for (int yy = 0; yy < 2; yy++)
			for (int xx = 0; xx < 2; xx++)
			{
				uint32_t wgt = wx[xx] * wy[yy];
				if (!wgt)
					continue;
				uint32_t tc = texel(src, t, level, xs[xx], ys[yy]);
				for (int k = 0; k < 4; k++)
					acc[k] += wgt * ((tc >> (8 * k)) & 0xffu);
			}
		for (int k = 0; k < 4; k++)
		{
			// roundEven(acc / 256)
			uint32_t q = acc[k] >> 8, r = acc[k] & 0xffu;
			if (r > 128 || (r == 128 && (q & 1)))
				q++;
			rgba[k] = q;
		}
	}

	// log2 for the LOD formula: ln m = 2 atanh((m - 1) / (m + 1)) by the series
	// s + s^3/3 + s^5/5 + s^7/7 + s^9/9 after reducing m to [sqrt(1/2), sqrt(2)];
	// one rounding per operation (the definition the CUDA sampler shares).
	static float lod_log2(float x)
	{
		uint32_t b;
		memcpy(&b, &x, 4);
		int32_t e = int32_t((b >> 23) & 0xffu) - 127;
		uint32_t mb = (b & 0x7fffffu) | 0x3f800000u;
		float m;
		memcpy(&m, &mb, 4);
		if (m > 1.41421356f)
		{
			m = m * 0.5f;
			e++;
		}
		float s = (m - 1.0f) / (m + 1.0f);
		float s2 = s * s;
		float poly = s2 * (1.0f / 9.0f);
		poly = poly + (1.0f / 7.0f);
		poly = s2 * poly;
		poly = poly + (1.0f / 5.0f);
		poly = s2 * poly;
		poly = poly + (1.0f / 3.0f);
		poly = s2 * poly;
		poly = poly + 1.0f;
		float ln_m = (2.0f * s) * poly;
		float l2 = ln_m * 1.44269504f;
		return float(e) + l2;
	}

	// sample_texture (gs/shaders/ubershader.comp:1042-1258): LOD from Q
	// (ceil(-log2|Q| * 2^(L+4) + K) / 16) or fixed (K >> 4), clamped to
	// [0, MXL]; MMIN applies when the LOD is positive; trilinear blends
	// floor(fract * 16) / 16 of the next level.  Levels past the texture's
	// chain read its last level.
	// Texel of layer `layer` of a super-sampled texture: layer 0 the
	// single-sampled texel, layer s + 1 sample s where the reference plane
	// marks it (upload.comp SUPER_SAMPLED, :131-220).
	uint32_t texel_layer(const uint8_t *src, const pgs_texture_desc &t, uint32_t layer, int32_t x, int32_t y)
	{
		if (layer == 0)
			return texel(src, t, 0, x, y);
		const uint32_t s = layer - 1;
		const uint32_t a = swizzle(uint32_t(x), uint32_t(y), t.tbp0, t.tbw, t.psm);
		switch (t.psm)
		{
		case CT24: case Z24:
		{
			uint32_t col = t32(src, 0, a), ref = t32(src, 1, a);
			if (ref != 0)
				col = (t32(src, 2 + s, a) & ref) | (col & ~ref);
			col &= 0xffffffu;
			uint32_t al = (t.aem && col == 0) ? 0 : t.ta0;
			return col | (al << 24);
		}
		case CT16: case CT16S: case Z16: case Z16S:
		{
			uint32_t c = t16(src, 0, a);
			if (t16(src, 1, a) == 0xffff)
				c = t16(src, 2 + s, a);
			uint32_t r = (c & 0x1f) << 3, g = ((c >> 5) & 0x1f) << 3, b = ((c >> 10) & 0x1f) << 3;
			uint32_t al = (t.aem && c == 0) ? 0 : ((c & 0x8000) ? t.ta1 : t.ta0);
			return r | (g << 8) | (b << 16) | (al << 24);
		}
		case T8:
		{
			uint32_t idx = t8(src, 0, a);
			if (t8(src, 1, a) == 0xff)
				idx = t8(src, 2 + s, a);
			return clut_color(t, idx);
		}
		case T8H:
		{
			uint32_t idx = t8(src, 0, 4 * a + 3);
			if (t8(src, 1, 4 * a + 3) == 0xff)
				idx = t8(src, 2 + s, 4 * a + 3);
			return clut_color(t, idx);
		}
		default:
		{
			uint32_t c = t32(src, 0, a);
			if (t32(src, 1, a) == 0xffffffffu)
				c = t32(src, 2 + s, a);
			return c;
		}
		}
	}

	static float average_sampling_offset(uint32_t rx, uint32_t ry)
	{
		// get_average_sampling_offset (utils.h:108-126).
		if (rx == ry)
		{
			const int rate = 1 << ry;
			return 0.5f * (float(rate - 1) / float(rate));
		}
		if (rx == 0 && ry == 1) return 0.25f;
		if (rx == 1 && ry == 2) return (0.125f + 0.625f) * 0.5f;
		if (rx == 0 && ry == 2) return 6.0f / 16.0f;
		if (rx == 1 && ry == 3) return (6.0f + 22.0f) / 64.0f;
		return 0.0f;
	}

	// Super-sampled texture sample (ubershader.comp:1155-1212): sample
	// mapping -> the shading sample's layer, resolved -> layer 0, otherwise
	// the phase LUT's taps around the texel below the sampling position with
	// unorm8 weights (one tap for nearest filtering or on a clamped region
	// edge); coordinates snap as for plain textures, taps wrap like them.
	void sample_layered(const PassCtx &, const uint8_t *src, const pgs_texture_desc &t, uint32_t tex_word, float u, float v,
	                    bool perspective, uint32_t sample, uint32_t rx, uint32_t ry, uint32_t rgba[4])
	{
		const bool clamp_s = tex_word & (1u << 19), clamp_t = tex_word & (1u << 20);
		const bool mag_linear = tex_word & (1u << 16);
		if (tex_word & ((1u << 25) | (1u << 26)))
		{
			const uint32_t layer = (tex_word & (1u << 25)) ? std::min(sample + 1, t.samples) : 0u;
			float w = float(1u << t.tw_log2), h = float(1u << t.th_log2);
			float uu = perspective ? u * w : u, vv = perspective ? v * h : v;
			if (clamp_s)
			{
				float lo = t.wms == 2 ? float(t.minu) : 0.0f, hi = t.wms == 2 ? float(t.maxu) : w - 1.0f;
				uu = std::min(std::max(uu, lo + 0.5f), hi + 0.5f);
			}
			if (clamp_t)
			{
				float lo = t.wmt == 2 ? float(t.minv) : 0.0f, hi = t.wmt == 2 ? float(t.maxv) : h - 1.0f;
				vv = std::min(std::max(vv, lo + 0.5f), hi + 0.5f);
			}
			float fu = uu * 16.0f;
			fu = fu + (1.0f / 64.0f);
			float fv = vv * 16.0f;
			fv = fv + (1.0f / 64.0f);
			const int32_t ku = int32_t(std::floor(fu)), kv = int32_t(std::floor(fv));
			if (!mag_linear)
			{
				uint32_t c = texel_layer(src, t, layer, wrap_coord(ku >> 4, t.wms, t.tw_log2, t.minu, t.maxu),
				                         wrap_coord(kv >> 4, t.wmt, t.th_log2, t.minv, t.maxv));
				for (int k = 0; k < 4; k++)
					rgba[k] = (c >> (8 * k)) & 0xffu;
				return;
			}
			const int32_t bu = ku - 8, bv = kv - 8;
			const int32_t x0 = bu >> 4, y0 = bv >> 4;
			const uint32_t fx = uint32_t(bu) & 15u, fy = uint32_t(bv) & 15u;
			const int32_t xs[2] = { wrap_coord(x0, t.wms, t.tw_log2, t.minu, t.maxu), wrap_coord(x0 + 1, t.wms, t.tw_log2, t.minu, t.maxu) };
			const int32_t ys[2] = { wrap_coord(y0, t.wmt, t.th_log2, t.minv, t.maxv), wrap_coord(y0 + 1, t.wmt, t.th_log2, t.minv, t.maxv) };
			const uint32_t wx[2] = { 16 - fx, fx }, wy[2] = { 16 - fy, fy };
			uint32_t acc[4] = { 0, 0, 0, 0 };
			for (int yy = 0; yy < 2; yy++)
				for (int xx = 0; xx < 2; xx++)
				{
					const uint32_t wgt = wx[xx] * wy[yy];
					if (!wgt)
						continue;
					const uint32_t c = texel_layer(src, t, layer, xs[xx], ys[yy]);
					for (int k = 0; k < 4; k++)
						acc[k] += wgt * ((c >> (8 * k)) & 0xffu);
				}
			for (int k = 0; k < 4; k++)
			{
				uint32_t q = acc[k] >> 8, r = acc[k] & 0xffu;
				if (r > 128 || (r == 128 && (q & 1)))
					q++;
				rgba[k] = q;
			}
			return;
		}
		const float w = float(1u << t.tw_log2), h = float(1u << t.th_log2);
		float uu = perspective ? u * w : u, vv = perspective ? v * h : v;
		const int32_t rx0 = t.wms == 2 ? int32_t(t.minu) : 0;
		const int32_t rx1 = t.wms == 2 ? int32_t(t.maxu) : (t.wms == 1 ? int32_t(w) - 1 : 0);
		const int32_t ry0 = t.wmt == 2 ? int32_t(t.minv) : 0;
		const int32_t ry1 = t.wmt == 2 ? int32_t(t.maxv) : (t.wmt == 1 ? int32_t(h) - 1 : 0);
		if (clamp_s)
			uu = std::min(std::max(uu, float(rx0) + 0.5f), float(rx1) + 0.5f);
		if (clamp_t)
			vv = std::min(std::max(vv, float(ry0) + 0.5f), float(ry1) + 0.5f);
		const float shift = 0.5f - average_sampling_offset(rx, ry);
		float su = uu + (1.0f / 1024.0f);
		su = su - shift;
		float sv = vv + (1.0f / 1024.0f);
		sv = sv - shift;
		const float fu = std::floor(su), fv = std::floor(sv);
		const int32_t ix = int32_t(fu), iy = int32_t(fv);
		const float pu = su - fu, pv = sv - fv;
		uint32_t entry, weights = 0;
		if (mag_linear)
		{
			const uint32_t lx = std::min(uint32_t(pu * 64.0f), 63u), ly = std::min(uint32_t(pv * 64.0f), 63u);
			entry = phase_lut[(ly * 64 + lx) * 2];
			weights = phase_lut[(ly * 64 + lx) * 2 + 1];
		}
		else
		{
			const uint32_t lx = std::min(uint32_t(pu * 32.0f), 31u), ly = std::min(uint32_t(pv * 32.0f), 31u);
			entry = phase_lut[64 * 64 * 2 + ly * 32 + lx];
		}
		const bool force_nearest = !mag_linear || ((clamp_s || clamp_t) && (ix == rx0 || iy == ry0 || ix == rx1 || iy == ry1));
		auto tap = [&](uint32_t layer, int32_t x, int32_t y) {
			return texel_layer(src, t, std::min(layer + 1, t.samples), wrap_coord(x, t.wms, t.tw_log2, t.minu, t.maxu),
			                   wrap_coord(y, t.wmt, t.th_log2, t.minv, t.maxv));
		};
		const uint32_t c0 = tap(entry & 15u, ix, iy);
		if (force_nearest)
		{
			for (int k = 0; k < 4; k++)
				rgba[k] = (c0 >> (8 * k)) & 0xffu;
			return;
		}
		uint32_t acc[4];
		for (int k = 0; k < 4; k++)
			acc[k] = (weights & 0xffu) * ((c0 >> (8 * k)) & 0xffu);
		for (uint32_t i = 1; i < 4; i++)
		{
			const uint32_t wi = (weights >> (8 * i)) & 0xffu;
			if (!wi)
				continue;
			int32_t ox = int32_t((entry >> (16 + 4 * i)) & 3u), oy = int32_t((entry >> (18 + 4 * i)) & 3u);
			if (ox >= 2) ox -= 4;
			if (oy >= 2) oy -= 4;
			const uint32_t c = tap((entry >> (4 * i)) & 15u, ix + ox, iy + oy);
			for (int k = 0; k < 4; k++)
				acc[k] += wi * ((c >> (8 * k)) & 0xffu);
		}
		for (int k = 0; k < 4; k++)
		{
			const uint32_t q = acc[k] / 255, r = acc[k] % 255;
			rgba[k] = q + (2 * r > 255 ? 1u : 0u);
		}
	}

	void sample_texture(const PassCtx &P, uint32_t tex_word, uint32_t tex2, float u, float v, float q,
	                    bool perspective, uint32_t sample, uint32_t rx, uint32_t ry, float out[4])
	{
		// Descriptors keep only the region modes; plain REPEAT and CLAMP come
		// from the primitive's sampler bits (TEX_SAMPLER_CLAMP_S/T,
		// gs/gs_interface.cpp:1514-1528, 1818-1820).
		pgs_texture_desc t = P.rp->textures[tex_word & 0xffffu];
		const uint8_t *src = P.tex_src[std::min<uint32_t>(tex_word & 0xffffu, P.rp->num_textures - 1)];
		if (t.wms < 2)
			t.wms = (tex_word & (1u << 19)) ? 1u : 0u;
		if (t.wmt < 2)
			t.wmt = (tex_word & (1u << 20)) ? 1u : 0u;
		if ((tex_word & (1u << 24)) && t.samples > 1)
		{
			uint32_t rgba[4];
			sample_layered(P, src, t, tex_word, u, v, perspective, sample, rx, ry, rgba);
			for (int k = 0; k < 4; k++)
				out[k] = float(rgba[k]);
			return;
		}
		bool clamp_s = tex_word & (1u << 19), clamp_t = tex_word & (1u << 20);
		bool mag_linear = tex_word & (1u << 16), min_linear = tex_word & (1u << 17);
		bool trilinear = tex_word & (1u << 18);
		uint32_t max_mip = (tex_word >> 21) & 7u;
		uint32_t rgba[4];
		if (max_mip == 0)
		{
			sample_level(src, t, 0, clamp_s, clamp_t, mag_linear, u, v, perspective, rgba);
		}
		else
		{
			int32_t K = int32_t((tex2 >> 3) & 0xfffu);
			if (K & 0x800)
				K -= 0x1000;
			float lod;
			bool linear;
			if (!(tex2 & 1u))
			{
				uint32_t L = (tex2 >> 1) & 3u;
				float aq = std::fabs(q), formula = 0.0f;
				if (std::isnormal(aq))
				{
					float scaled = -lod_log2(aq) * float(1u << (L + 4));
					formula = scaled + float(K);
				}
				lod = std::ceil(formula) * 0.0625f;
				linear = formula > 0.0f ? min_linear : mag_linear;
			}
			else
			{
				lod = float(K / 16 - ((K % 16) < 0 ? 1 : 0));
				linear = lod > 0.0f ? min_linear : mag_linear;
			}
			lod = std::min(std::max(lod, 0.0f), float(max_mip));
			float l1 = std::floor(lod), l2 = std::ceil(lod);
			uint32_t weight = uint32_t((lod - l1) * 16.0f);
			if (!trilinear)
			{
				weight = 0;
				l1 = float(int32_t(lod + 0.5f));
			}
			uint32_t last = std::max<uint32_t>(t.levels, 1) - 1;
			sample_level(src, t, std::min<uint32_t>(uint32_t(l1), last), clamp_s, clamp_t, linear, u, v, perspective, rgba);
			if (weight)
			{
				uint32_t c2[4];
				sample_level(src, t, std::min<uint32_t>(uint32_t(l2), last), clamp_s, clamp_t, linear, u, v, perspective,
				             c2);
				for (int k = 0; k < 4; k++)
				{
					uint32_t acc = (16 - weight) * rgba[k] + weight * c2[k];
					uint32_t r = acc / 16, f = acc % 16;
					if (f > 8 || (f == 8 && (r & 1)))
						r++;
					rgba[k] = r;
				}
			}
		}
		for (int k = 0; k < 4; k++)
			out[k] = float(rgba[k]);
	}

	// compute_combined_color (gs/shaders/ubershader.comp:1260-1339).
	void combined_color(const PassCtx &P, uint32_t pi, const Request &r, uint32_t combiner, float out[4],
	                    uint32_t sample_index)
	{
		const TAttr &a = P.tattr[pi];
		float col[4];
		for (int k = 0; k < 4; k++)
		{
			float c0 = unorm(a.rgba0, k), c1 = unorm(a.rgba1, k), c2 = unorm(a.rgba2, k);
			float t1 = (c1 - c0) * r.i;
			float t2 = c0 + t1;
			float t3 = (c2 - c0) * r.j;
			float t4 = t2 + t3;
			float t5 = 255.0f * t4;
			col[k] = std::floor(t5 + (1.0f / 256.0f));
		}
		bool fog = combiner & (1u << 3), tcc = combiner & (1u << 4), tme = combiner & (1u << 2);
		uint32_t mode = combiner & 3u;
		float cc[4];
		if (tme)
		{
			float stq[3];
			for (int k = 0; k < 3; k++)
			{
				float t1 = a.stqf1[k] * r.i;
				float t2 = a.stqf0[k] + t1;
				float t3 = a.stqf2[k] * r.j;
				stq[k] = t2 + t3;
			}
			float u = stq[0], v = stq[1];
			if (r.perspective && stq[2] != 1.0f)
			{
				u = u / stq[2];
				v = v / stq[2];
			}
			u = std::fmin(std::fmax(u, -2047.0f), 2047.0f);
			v = std::fmin(std::fmax(v, -2047.0f), 2047.0f);
			float tx[4];
			sample_texture(P, P.prims[pi].tex, P.prims[pi].tex2, u, v, stq[2], r.perspective, sample_index,
			               P.ss ? P.sr_x_log2 : 0u, P.ss ? P.sr_dim_log2 : 0u, tx);
			switch (mode)
			{
			case 1:
				memcpy(cc, tx, sizeof(cc));
				if (!tcc) cc[3] = col[3];
				break;
			case 0:
				for (int k = 0; k < 4; k++)
				{
					float m = col[k] * tx[k];
					m = m * (1.0f / 128.0f);
					cc[k] = std::min(std::max(std::floor(m), 0.0f), 255.0f);
				}
				if (!tcc) cc[3] = col[3];
				break;
			case 2:
			case 3:
				for (int k = 0; k < 4; k++)
				{
					float m = col[k] * tx[k];
					m = m * (1.0f / 128.0f);
					cc[k] = std::min(std::max(std::floor(m), 0.0f), 255.0f);
				}
				for (int k = 0; k < 3; k++)
					cc[k] += col[3];
				if (mode == 2)
					cc[3] = tcc ? tx[3] + col[3] : col[3];
				else
					cc[3] = tcc ? tx[3] : col[3];
				for (int k = 0; k < 4; k++)
					cc[k] = std::min(std::max(cc[k], 0.0f), 255.0f);
				break;
			}
		}
		else
			memcpy(cc, col, sizeof(cc));

		if (fog)
		{
			float t1 = a.stqf1[3] * r.i;
			float t2 = a.stqf0[3] + t1;
			float t3 = a.stqf2[3] * r.j;
			float f = round_even(t2 + t3);
			uint32_t fc = P.prims[pi].fogcol;
			for (int k = 0; k < 3; k++)
			{
				float fcol = unorm(fc, k) * 255.0f;
				float d = cc[k] - fcol;
				d = d * f;
				d = d * (1.0f / 256.0f);
				cc[k] = std::floor((fcol + d) + 0.5f);
			}
		}
		memcpy(out, cc, sizeof(cc));
	}

	// shade_resolve (gs/shaders/ubershader.comp:1464-1607) for one sample.
	void shade_resolve(const PassCtx &P, Sample &smp)
	{
		const Request &r = smp.pending;
		uint32_t pi = smp.pending_prim;
		const pgs_state_vector &sv = P.rp->states[r.state];
		bool zs = P.zb_psm != ~0u;
		bool z_pass = true;
		if (zs && r.z_test)
			z_pass = r.z_greater ? r.z > smp.depth : r.z >= smp.depth;
		if (!z_pass)
			return;

		float cc[4];
		combined_color(P, pi, r, sv.combiner, cc, P.ss ? smp.index : 0u);
		float fbc[4];
		for (int k = 0; k < 4; k++)
			fbc[k] = std::round(unorm(smp.color, k) * 255.0f);

		bool write_fb = true, write_zb = true, write_alpha = true;
		const pgs_primitive_attribute &pa = P.prims[pi];
		uint32_t bm = sv.blend_mode;
		bool ate = bm & (1u << 1);
		uint32_t atst = bfe(bm, 2, 3), afail = bfe(bm, 5, 2);
		bool date = bm & (1u << 7), datm = bm & (1u << 8);
		bool abe = bm & (1u << 9), pabe = bm & (1u << 10);
		bool colclamp = bm & (1u << 19), fba = bm & (1u << 20), dthe = bm & (1u << 21);
		bool fb24 = is24(P.fb_psm), fb32 = is32(P.fb_psm), fb16 = is16(P.fb_psm);

		if (P.has_aa1)
		{
			bool use_cov = (cc[3] == 128.0f || !abe) && r.multisample;
			if (use_cov)
				cc[3] = float(r.coverage);
			if (r.multisample)
				abe = true;
		}

		if (ate)
		{
			float aref = float(bfe(pa.alpha, 0, 8));
			float al = cc[3];
			bool pass;
			switch (atst)
			{
			case 0: pass = false; break;
			case 2: pass = al < aref; break;
			case 3: pass = al <= aref; break;
			case 4: pass = al == aref; break;
			case 5: pass = al >= aref; break;
			case 6: pass = al > aref; break;
			case 7: pass = al != aref; break;
			default: pass = true; break;
			}
			if (!pass)
			{
				switch (afail)
				{
				case 0: return;
				case 1: write_zb = false; break;
				case 2: write_fb = false; write_alpha = false; break;
				case 3: if (fb32) write_alpha = false; write_zb = false; break;
				}
			}
		}

		if (!fb24 && date)
		{
			uint32_t bit = fbc[3] >= 128.0f ? 1u : 0u;
			if (uint32_t(datm) != bit)
				return;
		}

		if (pabe && cc[3] < 128.0f)
			abe = false;

		float bl[4] = { cc[0], cc[1], cc[2], cc[3] };
		if (abe)
		{
			uint32_t am = bfe(bm, 11, 2), bmo = bfe(bm, 13, 2), cm = bfe(bm, 15, 2), dm = bfe(bm, 17, 2);
			float fix = float(bfe(pa.alpha, 8, 8));
			float C = 0.0f;
			if (cm == 0) C = cc[3];
			else if (cm == 1) C = fb24 ? 128.0f : fbc[3];
			else if (cm == 2) C = fix;
			for (int k = 0; k < 3; k++)
			{
				float A = am == 0 ? cc[k] : (am == 1 ? fbc[k] : 0.0f);
				float B = bmo == 0 ? cc[k] : (bmo == 1 ? fbc[k] : 0.0f);
				float D = dm == 0 ? cc[k] : (dm == 1 ? fbc[k] : 0.0f);
				float t = (A - B) * C;
				t = t * (1.0f / 128.0f);
				bl[k] = std::floor(t) + D;
			}
		}

		if (dthe)
		{
			int dim = int(P.sr_dim_log2);
			int px = (smp.hx >> dim) & 3, py = (smp.hy >> dim) & 3;
			int bit = ((py * 4 + px) * 4) & 31;
			uint32_t dimx = py < 2 ? sv.dimx_lo : sv.dimx_hi;
			int32_t dv = int32_t(bfe(dimx, bit, 3));
			dv = (dv << 29) >> 29; // bitfieldExtract on int sign-extends
			for (int k = 0; k < 3; k++)
				bl[k] += float(dv);
		}

		if (fb24) write_alpha = false;
		if (!write_alpha) bl[3] = fbc[3];
		if (!write_fb) { bl[0] = fbc[0]; bl[1] = fbc[1]; bl[2] = fbc[2]; }

		float out[4];
		for (int k = 0; k < 4; k++)
		{
			if (!colclamp)
			{
				float x = bl[k] / 256.0f;
				float fr = x - std::floor(x);
				out[k] = fr * (256.0f / 255.0f);
			}
			else
				out[k] = bl[k] * (1.0f / 255.0f);
		}
		uint32_t packed = pack_unorm(out);
		packed |= uint32_t(fba && write_alpha) << 31;

		uint32_t mask = pa.fbmsk;
		if (mask != ~0u && (write_fb || write_alpha))
		{
			if (mask != 0)
				smp.color = (packed & ~mask) | (smp.color & mask);
			else
				smp.color = packed;
			if (fb16)
				smp.color &= 0x80f8f8f8u;
			smp.color_dirty = true;
		}

		if (zs && write_zb && r.z_write)
		{
			smp.depth = r.z;
			smp.depth_dirty = true;
		}
	}

	void flush_pending(const PassCtx &P, Sample &smp)
	{
		if (smp.pending.coverage > 0)
			shade_resolve(P, smp);
		smp.pending.coverage = 0;
		smp.pending.z_write = false;
	}

	// Sample position within a pixel for a sampling pattern (get_tile_info,
	// gs/shaders/ubershader.comp:133-385, with 32-wide subgroups).
	static void sample_offset(uint32_t s, uint32_t xl, uint32_t yl, int32_t &ox, int32_t &oy)
	{
		uint32_t b0 = s & 1, b1 = (s >> 1) & 1, b2 = (s >> 2) & 1, b3 = (s >> 3) & 1;
		if (xl == yl)
		{
			ox = int32_t(b1 | (b3 << 1));
			oy = int32_t(b0 | (b2 << 1));
		}
		else if (yl == xl + 1)
		{
			// Checkerboard: local x is doubled and offset by local y parity.
			int32_t ly = int32_t(b0 | (xl >= 1 ? (b2 << 1) : 0));
			int32_t lx = int32_t(xl >= 1 ? b1 : 0);
			ox = (lx << 1) + (ly & 1);
			oy = ly;
		}
		else if (yl == xl + 2)
		{
			// Lanes: local y = bits 0-2, local x = bits 3-4; x is scaled by 4
			// and offset per row by bits (2 * (y & 3)) of 0x78 (:266-271, :333-338).
			int32_t ly = int32_t(s & ((1u << yl) - 1u));
			int32_t lx = int32_t(s >> yl);
			ox = (lx << 2) + int32_t((0x78u >> ((ly & 3) * 2)) & 3u);
			oy = ly;
		}
		else
		{
			ox = 0;
			oy = 0;
		}
	}

	void begin_sample(const PassCtx &P, Sample &smp, uint32_t sample_index, uint32_t fb_index, uint32_t z_index)
	{
		smp.color_dirty = false;
		smp.depth_dirty = false;
		uint32_t V16 = VRAM / 2, V32 = VRAM / 4;
		(void)V16; (void)V32;
		if (is16(P.fb_psm))
		{
			uint32_t col = w16(0, fb_index);
			if (P.ss)
			{
				uint32_t ref = w16(1, fb_index);
				if (ref == 0xffff)
					col = w16(2 + sample_index, fb_index);
			}
			smp.color = col_expand16(col);
		}
		else
		{
			smp.color = w32(0, fb_index);
			if (P.ss)
			{
				uint32_t ref = w32(1, fb_index);
				uint32_t rm = is24(P.fb_psm) ? 0xffffffu : ~0u;
				if ((ref & rm) == rm)
				{
					uint32_t sc = w32(2 + sample_index, fb_index);
					if (is24(P.fb_psm) && ref != ~0u)
						smp.color = (smp.color & 0xff000000u) | (sc & 0xffffffu);
					else
						smp.color = sc;
				}
			}
		}
		if (P.zb_psm != ~0u)
		{
			const uint8_t *zsrc = P.zcache ? P.zcache : vram.data();
			auto z16 = [&](uint32_t plane, uint32_t i) {
				uint16_t v;
				memcpy(&v, zsrc + plane * size_t(VRAM) + size_t(i) * 2, 2);
				return uint32_t(v);
			};
			auto z32 = [&](uint32_t plane, uint32_t i) {
				uint32_t v;
				memcpy(&v, zsrc + plane * size_t(VRAM) + size_t(i) * 4, 4);
				return v;
			};
			if (is16(P.zb_psm))
			{
				smp.depth = z16(0, z_index);
				if (P.ss && z16(1, z_index) == 0xffff)
					smp.depth = z16(2 + sample_index, z_index);
			}
			else
			{
				uint32_t rm = is24(P.zb_psm) ? 0xffffffu : ~0u;
				smp.depth = z32(0, z_index) & rm;
				if (P.ss && (z32(1, z_index) & rm) == rm)
					smp.depth = z32(2 + sample_index, z_index) & rm;
			}
		}
		else
			smp.depth = 0;
		smp.pending = Request();
	}

	static uint32_t col_expand16(uint32_t c)
	{
		uint32_t r = (c & 0x1f) << 3, g = ((c >> 5) & 0x1f) << 3, b = ((c >> 10) & 0x1f) << 3;
		uint32_t a = (c & 0x8000) ? 0x80u : 0u;
		return r | (g << 8) | (b << 16) | (a << 24);
	}

	// Shade one pixel with all its samples (main + end_tile).
	void shade_pixel(const PassCtx &P, int32_t px, int32_t py, const std::vector<uint32_t> &list)
	{
		uint32_t N = P.num_samples;
		Sample smp[16];
		uint32_t fb_index = swizzle(uint32_t(px), uint32_t(py), P.fb_base, P.fb_stride, P.fb_psm);
		uint32_t z_index = P.zb_psm != ~0u ? swizzle(uint32_t(px), uint32_t(py), P.zb_base, P.fb_stride, P.zb_psm) : 0;
		uint32_t D = P.sr_dim_log2;
		uint64_t covered = 0;

		for (uint32_t s = 0; s < N; s++)
		{
			int32_t ox = 0, oy = 0;
			if (P.ss)
				sample_offset(s, P.sr_x_log2, D, ox, oy);
			smp[s].hx = (px << D) + ox;
			smp[s].hy = (py << D) + oy;
			smp[s].index = s;
			begin_sample(P, smp[s], s, fb_index, z_index);

			Sample &S = smp[s];
			for (uint32_t pi : list)
			{
				bool opaque;
				Request px_req = shade_early(P, pi, S, opaque);
				if (px_req.coverage > 0)
				{
					covered++;
					if (px_req.z_test && !S.pending.z_write)
					{
						px_req.z_test = false;
						bool zp = px_req.z_greater ? px_req.z > S.depth : px_req.z >= S.depth;
						if (zp)
						{
							if (px_req.z_write && opaque)
							{
								px_req.z_write = false;
								S.depth = px_req.z;
								S.depth_dirty = true;
							}
						}
						else
						{
							px_req.coverage = 0;
							px_req.z_write = false;
						}
					}
					else if (px_req.z_write && !px_req.z_test && opaque)
					{
						px_req.z_write = false;
						S.pending.z_write = false;
						S.depth = px_req.z;
						S.depth_dirty = true;
					}
					bool affects = (px_req.z_test || !px_req.z_write) && S.pending.z_write;
					if (affects)
						opaque = false;
				}
				if (px_req.coverage > 0)
				{
					bool need_flush = !opaque && S.pending.coverage > 0;
					if (!need_flush)
					{
						S.pending = px_req;
						S.pending_prim = pi;
					}
					else
					{
						flush_pending(P, S);
						S.pending = px_req;
						S.pending_prim = pi;
					}
				}
			}
			flush_pending(P, S);
		}

		end_pixel(P, smp, N, fb_index, z_index);
		fragments.fetch_add(covered, std::memory_order_relaxed);
	}

	// end_tile (gs/shaders/ubershader.comp:581-780) for one pixel.
	void end_pixel(const PassCtx &P, Sample *smp, uint32_t N, uint32_t fb_index, uint32_t z_index)
	{
		bool zs = P.zb_psm != ~0u;
		bool req_color = false, req_depth = false;
		bool color_dirty = false, depth_dirty = false;
		for (uint32_t s = 0; s < N; s++)
		{
			color_dirty |= smp[s].color_dirty;
			depth_dirty |= smp[s].depth_dirty;
		}
		uint32_t color = smp[0].color;
		uint32_t depth = smp[0].depth;

		if (P.ss)
		{
			uint32_t first = smp[0].color;
			if (P.preserve_samples)
				req_color = true;
			else
				for (uint32_t s = 0; s < N; s++)
					req_color |= smp[s].color != first;
			if (zs)
				for (uint32_t s = 0; s < N; s++)
					req_depth |= smp[s].depth != smp[0].depth;

			if (req_color)
			{
				if (color_dirty)
					for (uint32_t s = 0; s < N; s++)
					{
						if (is16(P.fb_psm))
							w16(2 + s, fb_index) = uint16_t(((smp[s].color >> 3) & 0x1f) | (((smp[s].color >> 11) & 0x1f) << 5) |
							                                 (((smp[s].color >> 19) & 0x1f) << 10) | ((smp[s].color >> 31) << 15));
						else
							w32(2 + s, fb_index) = smp[s].color;
					}
				if (P.preserve_samples)
					color = first;
				else
				{
					float v[16][4];
					for (uint32_t s = 0; s < N; s++)
						for (int k = 0; k < 4; k++)
							v[s][k] = unorm(smp[s].color, k);
					for (uint32_t step = 8; step >= 1; step >>= 1)
					{
						if (step >= N)
							continue;
						float nv[16][4];
						for (uint32_t s = 0; s < N; s++)
							for (int k = 0; k < 4; k++)
								nv[s][k] = v[s][k] + v[s ^ step][k];
						memcpy(v, nv, sizeof(v));
					}
					float res[4];
					for (int k = 0; k < 4; k++)
						res[k] = v[0][k] / float(N);
					color = pack_unorm(res);
				}
			}

			if (zs && req_depth)
			{
				if (depth_dirty)
					for (uint32_t s = 0; s < N; s++)
					{
						if (is16(P.zb_psm))
							w16(2 + s, z_index) = uint16_t(smp[s].depth);
						else
							w32(2 + s, z_index) = smp[s].depth;
					}
				uint32_t m = smp[0].depth;
				for (uint32_t s = 1; s < N; s++)
					m = std::min(m, smp[s].depth);
				depth = m;
			}
		}

		if (color_dirty)
		{
			if (is16(P.fb_psm))
			{
				if (P.has_ss_reference)
					w16(1, fb_index) = req_color ? 0xffff : 0;
				w16(0, fb_index) = uint16_t(((color >> 3) & 0x1f) | (((color >> 11) & 0x1f) << 5) |
				                            (((color >> 19) & 0x1f) << 10) | ((color >> 31) << 15));
			}
			else
			{
				if (P.has_ss_reference)
					w32(1, fb_index) = req_color ? ~0u : 0u;
				w32(0, fb_index) = color;
			}
		}

		if (zs && depth_dirty)
		{
			if (is16(P.zb_psm))
			{
				if (P.has_ss_reference)
					w16(1, z_index) = req_depth ? 0xffff : 0;
				w16(0, z_index) = uint16_t(depth);
			}
			else
			{
				if (P.has_ss_reference)
					w32(1, z_index) = req_depth ? (is24(P.zb_psm) ? 0xffffffu : ~0u) : 0u;
				if (is24(P.zb_psm))
					w32(0, z_index) = (w32(0, z_index) & 0xff000000u) | (depth & 0xffffffu);
				else
					w32(0, z_index) = depth;
			}
		}
	}

	static uint32_t effective_z_psm(uint32_t color, uint32_t depth)
	{
		if (color == CT32 || color == CT24 || color == CT16S)
		{
			if (depth == CT32) return Z32;
			if (depth == CT24) return Z24;
			if (depth == CT16 || depth == CT16S) return Z16S;
		}
		else if (color == Z32 || color == Z24 || color == Z16S)
		{
			if (depth == Z32) return CT32;
			if (depth == Z24) return CT24;
			if (depth == Z16S || depth == Z16) return CT16S;
		}
		return depth;
	}

	// binning.comp update_heuristics (:87-125).
	static void heuristics(const pgs_primitive_attribute &pa, bool &req, bool &req_zw, bool &has_zw)
	{
		uint32_t s = pa.state;
		const uint32_t full_mask = (1u << 25) | (1u << 12) | (1u << 14);
		const uint32_t color_mask = (1u << 25) | (1u << 14);
		if ((s & full_mask) != color_mask) req_zw = true;
		if ((s & color_mask) != color_mask) req = true;
		if (s & (1u << 13)) has_zw = true;
		if (pa.tex & (1u << 24)) req = true;
	}

	// flush_rendering(rp, instance, base, count) (gs/gs_renderer.cpp:2919-3001).
	// Frame and depth buffer at the same base (GSRenderer::dispatch_shading,
	// gs/gs_renderer.cpp:2534-2650, dispatch_read_aliased_depth_passes
	// :2418-2487): primitives before the first depth-sensitive one render as
	// usual; while primitives write depth, one primitive at a time; after the
	// last depth write, in runs whose depth reads see a snapshot of VRAM taken
	// at the start of the run, a new run starting at each depth-tested sprite
	// that overlaps the run's area; with no depth reads left, as usual.
	void render_segment(PassCtx &P, uint32_t inst, uint32_t lo, uint32_t count)
	{
		const pgs_rp_instance &in = P.rp->instances[inst];
		const pgs_primitive_attribute *hp = P.rp->prims;
		const uint32_t end = lo + count;
		const uint32_t ZT = 1u << 12, ZW = 1u << 13, SPRITE = 1u << 21;
		P.zcache = nullptr;
		if (!in.z_sensitive || bfe(uint32_t(in.frame), 0, 9) != bfe(uint32_t(in.zbuf), 0, 9))
		{
			render_instance(P, inst, lo, count);
			return;
		}
		std::vector<uint32_t> mine;
		for (uint32_t i = lo; i < end; i++)
			if (bfe(hp[i].state, 29, 3) == inst)
				mine.push_back(i);
		int64_t first_zs = -1, last_zs = -1, last_zw = -1;
		for (uint32_t i : mine)
		{
			if (hp[i].state & ZW)
				last_zw = i;
			if (hp[i].state & (ZT | ZW))
			{
				if (first_zs < 0)
					first_zs = i;
				last_zs = i;
			}
		}
		if (first_zs < 0)
		{
			render_instance(P, inst, lo, count);
			return;
		}
		if (uint32_t(first_zs) > lo)
			render_instance(P, inst, lo, uint32_t(first_zs) - lo);
		uint32_t next = uint32_t(first_zs);
		if (last_zw >= 0)
		{
			for (uint32_t i : mine)
				if (int64_t(i) >= first_zs && int64_t(i) <= last_zw)
					render_instance(P, inst, i, 1);
			next = uint32_t(last_zw) + 1;
			if (next >= end)
				return;
			if (last_zs <= last_zw)
			{
				render_instance(P, inst, next, end - next);
				return;
			}
		}
		std::vector<uint8_t> snapshot;
		auto run_cached = [&](uint32_t a, uint32_t n) {
			snapshot.assign(vram.begin(), vram.end());
			P.zcache = snapshot.data();
			render_instance(P, inst, a, n);
			P.zcache = nullptr;
		};
		int32_t bx0 = INT32_MAX, by0 = INT32_MAX, bx1 = INT32_MIN, by1 = INT32_MIN;
		for (uint32_t i : mine)
		{
			if (i < next || !(hp[i].state & SPRITE))
				continue;
			const int16_t *pb = hp[i].bb;
			bool overlap = std::max<int32_t>(bx0, pb[0]) <= std::min<int32_t>(bx1, pb[2]) &&
			               std::max<int32_t>(by0, pb[1]) <= std::min<int32_t>(by1, pb[3]) &&
			               (hp[i].state & (ZT | ZW)) != 0;
			if (overlap)
			{
				if (i > next)
					run_cached(next, i - next);
				next = i;
				bx0 = pb[0]; by0 = pb[1]; bx1 = pb[2]; by1 = pb[3];
			}
			else
			{
				bx0 = std::min<int32_t>(bx0, pb[0]);
				by0 = std::min<int32_t>(by0, pb[1]);
				bx1 = std::max<int32_t>(bx1, pb[2]);
				by1 = std::max<int32_t>(by1, pb[3]);
			}
		}
		if (next < end)
			run_cached(next, end - next);
	}

	// render_pass_instance_might_field_render (gs/gs_renderer.cpp:1888-1895):
	// an instance that ends above row 256 may be a field; taller ones are
	// taken as full frames that are downsampled later.
	static bool might_field_render(const pgs_render_pass &rp, uint32_t instance)
	{
		const pgs_rp_instance &inst = rp.instances[instance];
		return !(inst.base_y + int32_t(inst.coarse_tiles_height << rp.coarse_tile_size_log2) > 256);
	}

	// Blend demotion budget (gs/gs_renderer.cpp:2082-2091): 32 primitives
	// per coarse tile when the hack is on and every state of the pass blends.
	static uint32_t blend_demote_budget(const pgs_render_pass &rp)
	{
		if (!rp.blend_demote)
			return 0;
		for (uint32_t i = 0; i < rp.num_states; i++)
			if ((rp.states[i].blend_mode & (1u << 9)) == 0)
				return 0;
		return 32;
	}

	void render_instance(PassCtx &P, uint32_t inst_index, uint32_t base, uint32_t count)
	{
		const pgs_rp_instance &inst = P.rp->instances[inst_index];
		uint32_t ts = P.rp->coarse_tile_size_log2;
		uint32_t fb_psm = bfe(uint32_t(inst.frame >> 24), 0, 6);
		uint32_t zpsm_raw = bfe(uint32_t(inst.zbuf >> 24), 0, 4) | 0x30u;
		P.fb_psm = fb_psm;
		P.fb_base = bfe(uint32_t(inst.frame), 0, 9) * 32;
		P.fb_stride = bfe(uint32_t(inst.frame), 16, 6);
		P.zb_base = bfe(uint32_t(inst.zbuf), 0, 9) * 32;
		P.zb_psm = inst.z_sensitive ? effective_z_psm(fb_psm, zpsm_raw) : ~0u;
		bool ss_inst = inst.sampling_rate_y_log2 != 0;
		const bool field_render = P.rp->field_aware && might_field_render(*P.rp, inst_index);
		const bool force_ss = field_render;
		const uint32_t blend_demote = blend_demote_budget(*P.rp);

		const int32_t ntiles = int32_t(inst.coarse_tiles_width * inst.coarse_tiles_height);
		const PassCtx shared = P;
		#pragma omp parallel for schedule(dynamic, 1)
		for (int32_t tile = 0; tile < ntiles; tile++)
		{
			PassCtx P = shared;
			uint32_t tx = uint32_t(tile) % inst.coarse_tiles_width, ty = uint32_t(tile) / inst.coarse_tiles_width;
			{
				int32_t lo0 = inst.base_x + int32_t(tx << ts), lo1 = inst.base_y + int32_t(ty << ts);
				int32_t hi0 = lo0 + (1 << ts) - 1, hi1 = lo1 + (1 << ts) - 1;
				std::vector<uint32_t> list;
				// Field rendering forces every covered tile super-sampled
				// (binning.comp:195, force_super_sample).
				bool req = force_ss, req_zw = false, has_zw = false;
				for (uint32_t p = base; p < base + count; p++)
				{
					if (bfe(P.prims[p].state, 29, 3) != inst_index)
						continue;
					bool ms_tri = bfe(P.prims[p].state, 16, 1) && !bfe(P.prims[p].state, 22, 1);
					if (intersects_tile(P.setup[p], lo0, lo1, hi0, hi1, ms_tri))
					{
						list.push_back(p);
						if (ss_inst)
							heuristics(P.prims[p], req, req_zw, has_zw);
					}
				}
				if (list.empty())
					continue;
				// Blend demotion: a tile crowded with blended primitives and no
				// depth writes shades single-sampled (binning.comp:277-282).
				if (blend_demote != 0 && list.size() >= blend_demote && !has_zw)
					req = false;
				req = req || (req_zw && has_zw);
				P.ss = ss_inst && req;
				if (P.ss)
				{
					P.sr_dim_log2 = inst.sampling_rate_y_log2;
					P.sr_x_log2 = inst.sampling_rate_x_log2;
					P.num_samples = 1u << (inst.sampling_rate_x_log2 + inst.sampling_rate_y_log2);
				}
				else
				{
					P.sr_dim_log2 = 0;
					P.sr_x_log2 = 0;
					P.num_samples = 1;
				}
				P.snap_mask_x = -(1 << inst.sampling_rate_y_log2);
				P.snap_mask_y = (inst.sampling_rate_y_log2 && field_render) ? (P.snap_mask_x >> 1) : P.snap_mask_x;
				P.preserve_samples = inst.channel_shuffle && inst.sampling_rate_y_log2 != 0;
				for (int32_t y = lo1; y <= hi1; y++)
					for (int32_t x = lo0; x <= hi0; x++)
						shade_pixel(P, x, y, list);
			}
		}
	}

	// Push constants of dispatch_triangle_setup / dispatch_single_sample_heuristic
	// (gs/gs_renderer.cpp:1914-1934, 1998-2036).
	struct HeuristicPush { uint32_t z_shift_bucket, z_shift, z_max; bool active; };

	static uint32_t heuristic_pushes(const pgs_render_pass *rp, HeuristicPush *push)
	{
		uint32_t packed = 0;
		HeuristicPush cur = {};
		for (uint32_t i = 0; i < rp->num_instances; i++)
		{
			const pgs_rp_instance &in = rp->instances[i];
			uint32_t depth_psm = in.z_sensitive ? (bfe(uint32_t(in.zbuf >> 24), 0, 4) | 0x30u) : 0x31u;
			if (depth_psm == 0x32 || depth_psm == 0x3a)
				packed |= 1u << (4 * i);
			else if (depth_psm == 0x31)
				packed |= 2u << (4 * i);
			else if (depth_psm == 0x30)
				packed |= 3u << (4 * i);
			if (in.sampling_rate_y_log2 == 0)
				continue;
			// Push constants persist across instances; an unknown format keeps
			// the previous values.
			if (depth_psm == 0x32 || depth_psm == 0x3a)
				cur = { 8, 0, 0xffffu, true };
			else if (depth_psm == 0x31)
				cur = { 16, 0, 0xffffffu, true };
			else if (depth_psm == 0x30)
				cur = { 16, 8, 0xffffffffu, true };
			push[i] = cur;
			push[i].active = true;
		}
		return packed;
	}

	static uint32_t hash_vertex(const pgs_vertex_position &v)
	{
		// single_sample_heuristic.comp:86-94.
		uint32_t s[3] = { uint32_t(v.x), uint32_t(v.y), v.z };
		for (int r = 0; r < 3; r++)
		{
			uint32_t t[3];
			for (int k = 0; k < 3; k++)
				t[k] = ((s[k] >> 8) ^ s[(k + 1) % 3]) * 1103515245u;
			s[0] = t[0]; s[1] = t[1]; s[2] = t[2];
		}
		return s[0] >> 16;
	}

	// single_sample_heuristic.comp:148-291, one workgroup per active bucket
	// and super-sampled instance.  All buckets read the states triangle setup
	// produced and the decisions are applied afterwards.  (The reference lets
	// workgroups see each other's writes; that only matters for a zero-area
	// primitive with unequal vertex depths, whose outcome there depends on
	// workgroup scheduling.)
	static void single_sample_heuristic(const pgs_render_pass *rp, std::vector<pgs_primitive_attribute> &prims,
	                                    const std::vector<int32_t> &bucket, const HeuristicPush *push)
	{
		const uint32_t n = rp->num_primitives;
		const pgs_vertex_position *vp = rp->positions;
		bool active_bucket[256] = {};
		for (uint32_t i = 0; i < n; i++)
			if (bucket[i] >= 0)
				active_bucket[bucket[i]] = true;
		std::vector<uint8_t> action(n, 0);
		const uint32_t SA = 1u << 26, SR = 1u << 25, LINE = 1u << 22, SPRITE = 1u << 21;
		const uint32_t NO_FULL_3D = SPRITE | LINE | SA;
		std::vector<uint8_t> full3d(65536), cand(65536), shared_v(65536);
		for (uint32_t inst = 0; inst < rp->num_instances; inst++)
		{
			if (!push[inst].active)
				continue;
			const HeuristicPush &h = push[inst];
			auto snap = [&](uint32_t z) { return std::min(h.z_max, z) >> h.z_shift; };
			for (uint32_t b = 0; b < 256; b++)
			{
				if (!active_bucket[b])
					continue;
				std::fill(full3d.begin(), full3d.end(), 0);
				std::fill(cand.begin(), cand.end(), 0);
				std::fill(shared_v.begin(), shared_v.end(), 0);
				bool any_full3d = false;
				uint32_t min_z = ~0u, max_z = 0;
				uint32_t zlo = b << h.z_shift_bucket, zhi = ((b + 1) << h.z_shift_bucket) - 1;
				auto in_range = [&](uint32_t s) { return s >= zlo && s <= zhi; };

				for (uint32_t i = 0; i < n; i++)
				{
					uint32_t st = prims[i].state;
					if (bfe(st, 29, 3) != inst)
						continue;
					if ((st & NO_FULL_3D) == 0)
					{
						for (int k = 0; k < 3; k++)
						{
							uint32_t z = vp[3 * i + k].z;
							min_z = std::min(min_z, z);
							max_z = std::max(max_z, z);
							uint32_t s = snap(z);
							if (in_range(s))
								full3d[s - zlo] = 1;
							any_full3d = true;
						}
					}
					else if ((st & (SA | SR)) == SA || (st & LINE))
					{
						uint32_t s = snap(vp[3 * i].z);
						if (in_range(s))
							cand[s - zlo] = 1;
					}
				}
				for (uint32_t i = 0; i < n; i++)
				{
					uint32_t st = prims[i].state;
					if (bfe(st, 29, 3) != inst || (st & NO_FULL_3D) != 0)
						continue;
					for (int k = 0; k < 3; k++)
					{
						uint32_t s = snap(vp[3 * i + k].z);
						if (in_range(s) && cand[s - zlo])
							shared_v[hash_vertex(vp[3 * i + k])] = 1;
					}
				}
				for (uint32_t i = 0; i < n; i++)
				{
					uint32_t st = prims[i].state;
					if (bfe(st, 29, 3) != inst || (st & (SA | SR)) != SA)
						continue;
					uint32_t s = snap(vp[3 * i].z);
					if (!in_range(s) || !full3d[s - zlo])
						continue;
					bool conflict = shared_v[hash_vertex(vp[3 * i])] || shared_v[hash_vertex(vp[3 * i + 1])] ||
					                shared_v[hash_vertex(vp[3 * i + 2])];
					if (conflict)
						cand[s - zlo] = 0;
				}
				bool force_single_sample = !any_full3d;
				for (uint32_t i = 0; i < n; i++)
				{
					uint32_t z = vp[3 * i].z;
					uint32_t s = snap(z);
					if (!in_range(s))
						continue;
					uint32_t st = prims[i].state;
					if (bfe(st, 29, 3) != inst)
						continue;
					bool tri = (st & (SA | SR)) == SA;
					bool line = force_single_sample && (st & LINE);
					if (!tri && !line)
						continue;
					if (cand[s - zlo])
						action[i] = 1;
					else if ((st & ((1u << 12) | (1u << 13))) && z > min_z && z < max_z)
						action[i] = 2;
				}
			}
		}
		for (uint32_t i = 0; i < n; i++)
		{
			if (action[i] == 1)
				prims[i].state |= SR;
			else if (action[i] == 2)
				prims[i].state &= ~SA;
		}
	}

	int flush_rendering(const pgs_render_pass *rp)
	{
		if (!rp)
			return 0;
		if (rp->num_primitives == 0)
		{
			snaps_taken = 0;
			return 0;
		}
		for (uint32_t i = 0; i < rp->num_textures; i++)
		{
			const pgs_texture_desc &d = rp->textures[i];
			if (d.levels > 7 || std::min(std::min(d.tw_log2, d.th_log2), 10u) + 1 < d.levels)
				return PGS_ERROR_INVALID_ARGUMENT;
			if (d.samples > 1 && (std::max<uint32_t>(d.levels, 1) != 1 || (d.samples & (d.samples - 1)) ||
			                      d.samples > 16 || 2 + d.samples > num_planes))
				return PGS_ERROR_INVALID_ARGUMENT;
		}
		std::vector<const uint8_t *> tex_src(std::max<uint32_t>(rp->num_textures, 1), nullptr);
		if (rp->num_textures)
		{
			// Plane 0, and every plane when super-sampled texture layers read
			// the reference plane and the samples.
			const size_t planes = rp->has_ss_textures ? num_planes : 1;
			tex_vram.assign(vram.begin(), vram.begin() + planes * size_t(VRAM));
			const uint32_t nsnap = std::min<uint32_t>(rp->num_snapshots, snaps_taken);
			for (uint32_t i = 0; i < rp->num_textures; i++)
			{
				tex_src[i] = tex_vram.data();
				for (uint32_t k = 0; k < nsnap; k++)
					if (i < rp->snapshot_textures[k])
					{
						tex_src[i] = snaps[k].data();
						break;
					}
			}
		}
		snaps_taken = 0;
		std::vector<pgs_primitive_attribute> prims(rp->prims, rp->prims + rp->num_primitives);
		std::vector<Setup> setup(rp->num_primitives);
		std::vector<TAttr> tattr(rp->num_primitives);
		PassCtx P = {};
		P.rp = rp;
		P.tex_src = tex_src.data();
		P.prims = prims.data();
		P.setup = setup.data();
		P.tattr = tattr.data();
		P.has_ss_reference = num_planes > 1;
		P.has_aa1 = rp->has_aa1;
		P.has_scanmsk = rp->has_scanmsk;
		P.tex_array = rp->has_ss_textures != 0;

		uint32_t fbmasks[8] = {};
		int srx = 0, sry = 0;
		for (uint32_t i = 0; i < rp->num_instances; i++)
		{
			fbmasks[i] = rp->instances[i].opaque_fbmask;
			srx = std::max<int>(srx, int(rp->instances[i].sampling_rate_x_log2));
			sry = std::max<int>(sry, int(rp->instances[i].sampling_rate_y_log2));
		}
		// render_pass_instance_is_deduced_blur (gs/gs_renderer.cpp:1850-1884):
		// an instance sampling one per-sample texture at two texel phases.
		uint32_t blur = 0;
		if (rp->num_primitives <= 64)
			for (uint32_t inst = 0; inst < rp->num_instances; inst++)
			{
				uint32_t last = ~0u;
				int32_t ph0 = 0, ph1 = 0;
				for (uint32_t i = 0; i < rp->num_primitives; i++)
				{
					const pgs_primitive_attribute &pa = rp->prims[i];
					if (bfe(pa.state, 29, 3) != inst || !(pa.tex & (1u << 24)))
						continue;
					if (pa.state & (1u << 18))
						break;
					const uint32_t ti = pa.tex & 0xffffu;
					const int32_t a0 = int32_t(rp->attributes[3 * i].u) - rp->positions[3 * i].x;
					const int32_t a1 = int32_t(rp->attributes[3 * i].v) - rp->positions[3 * i].y;
					if (last == ti)
					{
						if (a0 != ph0 || a1 != ph1)
						{
							blur |= 1u << inst;
							break;
						}
					}
					else
					{
						ph0 = a0;
						ph1 = a1;
					}
					last = ti;
				}
			}
		// FORCE_LINEAR_SUPER_SAMPLE (gs/gs_renderer.cpp:1953-1969): field
		// rendering with super-sampled textures bound.
		bool force_linear = false;
		if (rp->has_ss_textures && rp->field_aware)
			for (uint32_t inst = 0; inst < rp->num_instances; inst++)
				force_linear = force_linear || might_field_render(*rp, inst);
		HeuristicPush push[8] = {};
		uint32_t packed_z_shift = heuristic_pushes(rp, push);
		std::vector<int32_t> bucket(rp->num_primitives);
		#pragma omp parallel for schedule(static)
		for (uint32_t i = 0; i < rp->num_primitives; i++)
			triangle_setup(i, rp->positions, rp->attributes, prims[i], setup[i], tattr[i], fbmasks, srx, sry,
			               packed_z_shift, bucket[i], rp, blur, force_linear);
		if (sry != 0)
			single_sample_heuristic(rp, prims, bucket, push);
		for (uint32_t i = 0; i < rp->num_primitives; i++)
			state_log.push_back(prims[i].state);

		// Instance ordering (gs/gs_renderer.cpp:3190-3266).
		if (rp->num_instances == 1)
		{
			render_segment(P, 0, 0, rp->num_primitives);
			return 0;
		}
		uint8_t hazard[8] = {};
		bool any = false;
		compute_hazards(rp, hazard, any);
		if (any)
		{
			uint32_t active = 0, active_h = 0, base = 0;
			for (uint32_t p = 0; p < rp->num_primitives; p++)
			{
				uint32_t inst = bfe(P.prims[p].state, 29, 3);
				if (active_h & (1u << inst))
				{
					for (uint32_t b = 0; b < 8; b++)
						if (active & (1u << b))
							render_segment(P, b, base, p - base);
					base = p;
					active = 0;
					active_h = 0;
				}
				active |= 1u << inst;
				active_h |= hazard[inst];
			}
			for (uint32_t b = 0; b < 8; b++)
				if (active & (1u << b))
					render_segment(P, b, base, rp->num_primitives - base);
		}
		else
		{
			uint32_t lo[8], hi[8];
			for (int i = 0; i < 8; i++) { lo[i] = ~0u; hi[i] = 0; }
			for (uint32_t p = 0; p < rp->num_primitives; p++)
			{
				uint32_t inst = bfe(P.prims[p].state, 29, 3);
				if (lo[inst] == ~0u) lo[inst] = p;
				hi[inst] = p;
			}
			for (uint32_t i = 0; i < rp->num_instances; i++)
				if (lo[i] != ~0u)
					render_segment(P, i, lo[i], hi[i] - lo[i] + 1);
		}
		return 0;
	}

	struct PR { uint32_t start, end; };

	static PR page_range(uint32_t base_block, int32_t x, int32_t y, uint32_t w, uint32_t h, uint32_t stride, uint32_t psm)
	{
		Geo g = geometry(psm);
		if (psm == T4 || psm == T8) stride >>= 1;
		uint32_t px0 = uint32_t(x) / g.page_w, px1 = (uint32_t(x) + w - 1) / g.page_w;
		uint32_t py0 = uint32_t(y) / g.page_h, py1 = (uint32_t(y) + h - 1) / g.page_h;
		uint32_t base = base_block / 32;
		uint32_t s = base + py0 * stride + px0;
		uint32_t e = base + py1 * stride + px1 + ((base_block % 32) ? 1 : 0);
		return { s, e };
	}

	// compute_instance_hazard_mask (gs/gs_renderer.cpp:3034-3075).
	static void compute_hazards(const pgs_render_pass *rp, uint8_t *mask, bool &any)
	{
		PR fb[8], zb[8];
		uint32_t ts = rp->coarse_tile_size_log2;
		for (uint32_t i = 0; i < rp->num_instances; i++)
		{
			auto &in = rp->instances[i];
			uint32_t fbp = bfe(uint32_t(in.frame), 0, 9), fbw = bfe(uint32_t(in.frame), 16, 6);
			uint32_t fpsm = bfe(uint32_t(in.frame >> 24), 0, 6);
			fb[i] = page_range(fbp * 32, in.base_x, in.base_y, in.coarse_tiles_width << ts, in.coarse_tiles_height << ts, fbw, fpsm);
			if (in.z_sensitive)
			{
				uint32_t zbp = bfe(uint32_t(in.zbuf), 0, 9), zpsm = bfe(uint32_t(in.zbuf >> 24), 0, 4);
				zb[i] = page_range(zbp * 32, in.base_x, in.base_y, in.coarse_tiles_width << ts, in.coarse_tiles_height << ts, fbw, zpsm);
			}
		}
		auto ov = [](PR a, PR b) { return std::max(a.start, b.start) <= std::min(a.end, b.end); };
		any = false;
		for (uint32_t i = 0; i < rp->num_instances; i++)
			for (uint32_t j = i + 1; j < rp->num_instances; j++)
			{
				auto &a = rp->instances[i], &b = rp->instances[j];
				bool h = ov(fb[i], fb[j]) || (b.z_sensitive && ov(fb[i], zb[j])) || (a.z_sensitive && ov(fb[j], zb[i])) ||
				         (a.z_sensitive && b.z_sensitive && (a.z_write || b.z_write) && ov(zb[i], zb[j]));
				if (h)
				{
					mask[i] |= uint8_t(1u << j);
					mask[j] |= uint8_t(1u << i);
					any = true;
				}
			}
	}

	// -----------------------------------------------------------------------
	// vram_copy.comp (HOST_TO_LOCAL and LOCAL_TO_LOCAL), sequential.
	void write_pixel(uint32_t psm, uint32_t addr, uint32_t data)
	{
		bool inv = num_planes > 1;
		if (is24(psm))
		{
			uint32_t &w = w32(0, addr);
			w = (w & 0xff000000u) | (data & 0xffffffu);
			if (inv) { uint32_t &r = w32(1, addr); r &= 0xff000000u; }
		}
		else if (is16(psm))
		{
			w16(0, addr) = uint16_t(data);
			if (inv) w16(1, addr) = 0;
		}
		else if (psm == T8)
		{
			w8(0, addr) = uint8_t(data);
			if (inv) w8(1, addr) = 0;
		}
		else if (psm == T8H)
		{
			w8(0, addr * 4 + 3) = uint8_t(data);
			if (inv) w8(1, addr * 4 + 3) = 0;
		}
		else if (psm == T4)
		{
			uint8_t &b = w8(0, addr >> 1);
			uint32_t sh = (addr & 1) * 4;
			b = uint8_t((b & ~(0xfu << sh)) | ((data & 0xfu) << sh));
			if (inv) { uint8_t &r = w8(1, addr >> 1); r = uint8_t(r & ~(0xfu << sh)); }
		}
		else if (psm == T4HL || psm == T4HH)
		{
			uint32_t sh = psm == T4HL ? 24 : 28;
			uint32_t &w = w32(0, addr);
			w = (w & ~(0xfu << sh)) | ((data & 0xfu) << sh);
			if (inv) { uint32_t &r = w32(1, addr); r &= ~(0xfu << sh); }
		}
		else
		{
			w32(0, addr) = data;
			if (inv) w32(1, addr) = 0;
		}
	}

	uint32_t read_pixel(uint32_t psm, uint32_t addr)
	{
		if (is16(psm)) return w16(0, addr);
		if (psm == T8) return w8(0, addr);
		if (psm == T8H) return w8(0, addr * 4 + 3);
		if (psm == T4) return (w8(0, addr >> 1) >> ((addr & 1) * 4)) & 15u;
		if (psm == T4HL) return (w32(0, addr) >> 24) & 15u;
		if (psm == T4HH) return w32(0, addr) >> 28;
		return w32(0, addr);
	}

	int copy_vram(const pgs_copy_desc *d)
	{
		uint64_t bb = d->bitbltbuf;
		uint32_t sbp = bfe(uint32_t(bb), 0, 14), sbw = bfe(uint32_t(bb), 16, 6), spsm = bfe(uint32_t(bb), 24, 6);
		uint32_t dbp = bfe(uint32_t(bb >> 32), 0, 14), dbw = bfe(uint32_t(bb >> 32), 16, 6), dpsm = bfe(uint32_t(bb >> 32), 24, 6);
		uint32_t ssax = bfe(uint32_t(d->trxpos), 0, 11), ssay = bfe(uint32_t(d->trxpos), 16, 11);
		uint32_t dsax = bfe(uint32_t(d->trxpos >> 32), 0, 11), dsay = bfe(uint32_t(d->trxpos >> 32), 16, 11);
		uint32_t w = bfe(uint32_t(d->trxreg), 0, 12), h = bfe(uint32_t(d->trxreg >> 32), 0, 12);
		uint32_t xdir = bfe(uint32_t(d->trxdir), 0, 2);
		if (w == 0 || h == 0)
			return 0;

		uint32_t eff_stride = dbw;
		if (dpsm == T4 || dpsm == T8)
			eff_stride &= ~1u;
		Geo g = geometry(dpsm);

		if (xdir == 0)
		{
			const uint8_t *src = static_cast<const uint8_t *>(d->host_data);
			uint64_t size = d->host_size;
			uint64_t off_q = d->host_offset / 8;
			uint32_t b = bpp(dpsm);
			for (uint32_t y = 0; y < h; y++)
				for (uint32_t x = 0; x < w; x++)
				{
					if (x >= eff_stride * 64)
					{
						uint32_t last = (dsay + h - 1) / g.page_h, cur = (dsay + y) / g.page_h;
						if (last != cur)
							continue;
					}
					// Partial-flush skip and availability tests exactly as written in
					// vram_copy.comp:326-330,354-358,391-395,437-441 and :549-553.
					uint64_t sa = uint64_t(y) * w + x;
					uint64_t factor = (b == 32 || b == 24) ? 2 : (b == 16 ? 4 : (b == 8 ? 8 : 16));
					uint64_t avail = b == 32 ? size / 4 : (b == 24 ? size / 3 : (b == 16 ? size / 2 : (b == 8 ? size : 2 * size)));
					if (sa * factor < off_q)
						continue;
					if (sa >= avail)
						continue;
					uint32_t data;
					if (b == 24) data = src[3 * sa] | (src[3 * sa + 1] << 8) | (src[3 * sa + 2] << 16);
					else if (b == 16) { uint16_t v; memcpy(&v, src + 2 * sa, 2); data = v; }
					else if (b == 8) data = src[sa];
					else if (b == 4) data = (src[sa >> 1] >> ((sa & 1) * 4)) & 15u;
					else memcpy(&data, src + 4 * sa, 4);
					uint32_t dx = (x + dsax) & 2047, dy = (y + dsay) & 2047;
					write_pixel(dpsm, swizzle(dx, dy, dbp, dbw, dpsm), data);
				}
		}
		else if (xdir == 2)
		{
			// Local copies read the source as it was before the copy.
			std::vector<uint8_t> snapshot(vram.begin(), vram.begin() + VRAM);
			auto rd = [&](uint32_t psm, uint32_t a) -> uint32_t {
				const uint8_t *v = snapshot.data();
				uint32_t r32, r16;
				if (is16(psm)) { memcpy(&r16, v + 2 * a, 2); return r16 & 0xffffu; }
				if (psm == T8) return v[a];
				if (psm == T8H) return v[4 * a + 3];
				if (psm == T4) return (v[a >> 1] >> ((a & 1) * 4)) & 15u;
				memcpy(&r32, v + 4 * a, 4);
				if (psm == T4HL) return (r32 >> 24) & 15u;
				if (psm == T4HH) return r32 >> 28;
				return r32;
			};
			for (uint32_t y = 0; y < h; y++)
				for (uint32_t x = 0; x < w; x++)
				{
					if (x >= eff_stride * 64)
					{
						uint32_t last = (dsay + h - 1) / g.page_h, cur = (dsay + y) / g.page_h;
						if (last != cur)
							continue;
					}
					uint32_t sx = (x + ssax) & 2047, sy = (y + ssay) & 2047;
					uint32_t dx = (x + dsax) & 2047, dy = (y + dsay) & 2047;
					uint32_t data = rd(spsm, swizzle(sx, sy, sbp, sbw, spsm));
					write_pixel(dpsm, swizzle(dx, dy, dbp, dbw, dpsm), data);
				}
		}
		return 0;
	}

	// -----------------------------------------------------------------------
	// clut_write.comp.
	int update_palette(const pgs_palette_upload *u)
	{
		uint32_t inst = u->target ? (u->target - 1u) % PGS_CLUT_INSTANCES : (last_clut_instance + 1) % PGS_CLUT_INSTANCES;
		last_clut_instance = inst;
		uint16_t tmp[512];
		memcpy(tmp, &clut[size_t(u->base_instance) * 512], sizeof(tmp));
		uint64_t t = u->tex0;
		uint32_t psm = uint32_t((t >> 20) & 0x3f);
		uint32_t cbp = uint32_t((t >> 37) & 0x3fff);
		uint32_t cpsm = uint32_t((t >> 51) & 0xf);
		uint32_t csm = uint32_t((t >> 55) & 1);
		uint32_t csa = uint32_t((t >> 56) & 0x1f);
		uint32_t cbw = bfe(uint32_t(u->texclut), 0, 6), cou = bfe(uint32_t(u->texclut), 6, 6), cov = bfe(uint32_t(u->texclut), 12, 10);
		bool index4 = psm == T4 || psm == T4HH || psm == T4HL;
		for (uint32_t lane = 0; lane < 256; lane++)
		{
			bool active;
			uint32_t wc = lane + csa * 16, rc = lane;
			if (index4)
				active = lane < 16;
			else if (csm == 0)
			{
				uint32_t csa_count = cpsm == CT32 ? 16u : 32u;
				uint32_t active_csa = csa_count - csa;
				active = lane < active_csa * 16;
				rc += csa * 16;
			}
			else
				active = true;
			if (!active)
				continue;
			uint32_t cx, cy;
			if (csm != 0)
			{
				cx = uint32_t(float(rc) * u->csm2_x_scale + 1.0f / 256.0f) + u->csm2_x_bias + cou * 16;
				cy = cov;
			}
			else
			{
				cx = (rc & 7) | (((rc >> 4) & 1) << 3);
				cy = ((rc >> 3) & 1) | (((rc >> 5) & 7) << 1);
			}
			if (cpsm == CT32)
			{
				uint32_t v = w32(0, swizzle(cx, cy, cbp, cbw, CT32));
				if (wc < 512) tmp[wc] = uint16_t(v);
				if (wc + 256 < 512) tmp[wc + 256] = uint16_t(v >> 16);
			}
			else
			{
				uint32_t v = w16(0, swizzle(cx, cy, cbp, cbw, cpsm));
				if (wc < 512) tmp[wc] = uint16_t(v);
			}
		}
		memcpy(&clut[size_t(inst) * 512], tmp, sizeof(tmp));
		return int(inst);
	}

	// GSRenderer::init_phase_lut (gs/gs_renderer.cpp:93-315): per 64 x 64
	// sub-texel phase the four nearest sampling-grid points (sample id, texel
	// offset in -1..1), the first in the centre texel, with tent weights over
	// the falloff distance quantised to unorm8 summing to 255; per 32 x 32 phase
	// the nearest sample.  Equal distances keep generation order.
	void init_phase_lut(uint32_t rx, uint32_t ry)
	{
		std::fill(std::begin(phase_lut), std::end(phase_lut), 0u);
		if (!rx && !ry)
			return;
		const int G = 64, n = 1 << (rx + ry);
		struct Pt { int x, y; };
		auto grid = [&](std::vector<Pt> &pts, bool nearest) {
			pts.resize(n);
			for (int i = 0; i < n; i++)
			{
				Pt q;
				if (int(ry) - int(rx) == 2)
				{
					const int sparse[4] = { 0, 2, 3, 1 };
					q = { (i / 8) * 4 + sparse[i % 4], i % 8 };
				}
				else
				{
					q.y = ((i >> 0) & 1) + ((i >> 2) & 1) * 2;
					q.x = ((i >> 1) & 1) + ((i >> 3) & 1) * 2;
					if (int(ry) - int(rx) == 1)
						q.x = q.x * 2 + i % 2;
				}
				const int scale = G >> ry;
				q.x *= scale;
				q.y *= scale;
				if (nearest)
				{
					q.x += (scale - 1) >> 1;
					q.y += (scale - 1) >> 1;
				}
				pts[i] = q;
			}
		};
		struct R { int sample, tx, ty, dx, dy, m; };
		auto near = [&](int x, int y, const std::vector<Pt> &pts, int sup, std::vector<R> &res) {
			res.clear();
			for (int i = 0; i < n; i++)
				for (int ty = -sup; ty <= sup; ty++)
					for (int tx = -sup; tx <= sup; tx++)
					{
						int dx = std::abs(pts[i].x + G * tx - x), dy = std::abs(pts[i].y + G * ty - y);
						res.push_back({ i, tx, ty, dx, dy, std::max(dx, dy) });
					}
			std::stable_sort(res.begin(), res.end(),
			                 [](const R &a, const R &b) { return a.m == b.m ? a.dy < b.dy : a.m < b.m; });
		};
		std::vector<Pt> pts, pts_n;
		grid(pts, false);
		grid(pts_n, true);
		std::vector<R> res;
		int falloff = INT32_MAX;
		for (int y = 0; y < G; y++)
			for (int x = 0; x < G; x++)
			{
				near(x, y, pts, 1, res);
				falloff = std::min(falloff, res[4].m);
			}
		for (int y = 0; y < G; y++)
			for (int x = 0; x < G; x++)
			{
				near(x, y, pts, 1, res);
				if (res[0].tx != 0 || res[0].ty != 0)
					for (size_t i = 1; i < res.size(); i++)
						if (res[i].tx == 0 && res[i].ty == 0)
						{
							if (i < 4)
								std::swap(res[0], res[i]);
							else
							{
								std::swap(res[3], res[i]);
								std::swap(res[0], res[3]);
							}
							break;
						}
				uint32_t ex = 0, ey = 0, total = 0;
				float wt[4], sum = 0.0f;
				for (int i = 0; i < 4; i++)
				{
					ex |= uint32_t(res[i].sample) << (4 * i);
					ex |= (uint32_t(res[i].tx) & 3u) << (4 * i + 16);
					ex |= (uint32_t(res[i].ty) & 3u) << (4 * i + 18);
					float fx = float(res[i].dx) / float(falloff), fy = float(res[i].dy) / float(falloff);
					wt[i] = std::max(0.0f, 1.0f - fx) * std::max(0.0f, 1.0f - fy);
					sum += wt[i];
				}
				if (sum < 0.001f)
				{
					for (float &v : wt)
						v = 1.0f;
					sum = 4.0f;
				}
				for (int i = 0; i < 3; i++)
				{
					float sc = wt[i] * 255.0f / sum;
					uint32_t q = std::min<uint32_t>(uint32_t(sc + 0.5f), 255u - total);
					total += q;
					ey |= q << (8 * i);
				}
				ey |= (255u - total) << 24;
				phase_lut[(y * G + x) * 2] = ex;
				phase_lut[(y * G + x) * 2 + 1] = ey;
			}
		for (int y = 0; y < G / 2; y++)
			for (int x = 0; x < G / 2; x++)
			{
				near(2 * x, 2 * y, pts_n, 0, res);
				phase_lut[G * G * 2 + y * (G / 2) + x] = uint32_t(res[0].sample);
			}
	}

	int set_ss(uint32_t x, uint32_t y)
	{
		init_phase_lut(x, y);
		rate_x = x;
		rate_y = y;
		uint32_t planes = (x | y) ? 2u + (1u << (x + y)) : 1u;
		if (planes != num_planes)
		{
			std::vector<uint8_t> n(size_t(planes) * VRAM, 0);
			memcpy(n.data(), vram.data(), VRAM);
			vram.swap(n);
			num_planes = planes;
		}
		else if (planes > 1)
			memset(vram.data() + VRAM, 0, size_t(planes - 1) * VRAM);
		return 0;
	}
};
} // namespace oracle

// ---------------------------------------------------------------------------
// pgs_backend_ops table.
using oracle::Backend;

static void o_destroy(void *self) { delete static_cast<Backend *>(self); }
static int o_reserve(void *self, uint32_t n, pgs_vertex_position **p, pgs_vertex_attribute **a, pgs_primitive_attribute **pr)
{
	auto *b = static_cast<Backend *>(self);
	if (n > PGS_MAX_PRIMITIVES_PER_FLUSH)
		return PGS_ERROR_INVALID_ARGUMENT;
	*p = b->res_pos.data();
	*a = b->res_attr.data();
	*pr = b->res_prim.data();
	return 0;
}
static int o_flush_rendering(void *self, const pgs_render_pass *rp) { return static_cast<Backend *>(self)->flush_rendering(rp); }
static int o_copy(void *self, const pgs_copy_desc *d) { return static_cast<Backend *>(self)->copy_vram(d); }
static int o_palette(void *self, const pgs_palette_upload *u) { return static_cast<Backend *>(self)->update_palette(u); }
static int o_set_ss(void *self, uint32_t x, uint32_t y) { return static_cast<Backend *>(self)->set_ss(x, y); }
static int o_snapshot(void *self)
{
	auto *b = static_cast<Backend *>(self);
	if (b->snaps_taken >= PGS_MAX_VRAM_SNAPSHOTS)
		return PGS_ERROR_CAPACITY;
	b->snaps[b->snaps_taken].assign(b->vram.begin(), b->vram.end());
	return int(b->snaps_taken++);
}
static int o_submit(void *) { return 0; }
static int o_read(void *self, uint32_t plane, uint64_t off, uint64_t size, void *dst)
{
	auto *b = static_cast<Backend *>(self);
	if (plane >= b->num_planes || off + size > oracle::VRAM)
		return PGS_ERROR_INVALID_ARGUMENT;
	memcpy(dst, b->vram.data() + size_t(plane) * oracle::VRAM + off, size);
	return 0;
}
static int o_write(void *self, uint64_t off, uint64_t size, const void *src)
{
	auto *b = static_cast<Backend *>(self);
	if (off + size > oracle::VRAM)
		return PGS_ERROR_INVALID_ARGUMENT;
	memcpy(b->vram.data() + off, src, size);
	if (b->num_planes > 1)
		memset(b->vram.data() + oracle::VRAM + off, 0, size);
	return 0;
}
static int o_error(void *, uint32_t *flags) { if (flags) *flags = 0; return 0; }

// sample_circuit.frag:51-148: one circuit read-out from the current VRAM
// planes.  16-bit texels expand with alpha 0 / 0xff (rgba16_to_rgba32 with
// TA0 = 0, TA1 = 0xff); 32-bit formats other than CT32 read alpha as 0x80.
static uint32_t circuit_payload(const std::vector<uint8_t> &vram, uint32_t psm, uint32_t addr, uint32_t plane)
{
	const bool is16 = psm == 0x02 || psm == 0x0a || psm == 0x32 || psm == 0x3a;
	if (is16)
	{
		uint16_t v;
		memcpy(&v, vram.data() + size_t(plane) * oracle::VRAM + size_t(addr) * 2, 2);
		uint32_t r = (v & 0x1fu) << 3, g = ((v >> 5) & 0x1fu) << 3, b = ((v >> 10) & 0x1fu) << 3;
		uint32_t a = (v & 0x8000u) ? 0xffu : 0u;
		return r | (g << 8) | (b << 16) | (a << 24);
	}
	uint32_t v;
	memcpy(&v, vram.data() + size_t(plane) * oracle::VRAM + size_t(addr) * 4, 4);
	if (psm != 0x00)
		v = (v & ~0xff000000u) | 0x80000000u;
	return v;
}

static int o_circuit(void *self, const pgs_circuit_params *cp, void *dst)
{
	if (!cp || !dst)
		return PGS_ERROR_INVALID_ARGUMENT;
	const pgs_circuit_params &C = *cp;
	auto *b = static_cast<Backend *>(self);
	if (C.super_samples > 1 && 2u + C.super_samples > b->num_planes)
		return PGS_ERROR_INVALID_ARGUMENT;
	const bool is16 = C.psm == 0x02 || C.psm == 0x0a || C.psm == 0x32 || C.psm == 0x3a;
	uint32_t *out = static_cast<uint32_t *>(dst);
	for (uint32_t y = 0; y < C.height; y++)
		for (uint32_t x = 0; x < C.width; x++)
		{
			uint32_t o = 0;
			if (x < C.valid_width && y < C.valid_height)
			{
				uint32_t sx = C.super_samples >= 4 ? x >> 1 : x, sy = C.super_samples >= 4 ? y >> 1 : y;
				uint32_t cx = sx + C.dbx, cy = sy * C.phase_stride + C.dby + C.phase;
				uint32_t addr = oracle::swizzle(cx, cy, C.fbp * 32, C.fbw, C.psm);
				bool valid = false;
				if (C.super_samples >= 4)
				{
					if (is16)
					{
						uint16_t r;
						memcpy(&r, b->vram.data() + oracle::VRAM + size_t(addr) * 2, 2);
						valid = r == 0xffff;
					}
					else
					{
						uint32_t r;
						memcpy(&r, b->vram.data() + oracle::VRAM + size_t(addr) * 4, 4);
						valid = C.psm != 0x00 ? (r & 0xffffffu) == 0xffffffu : r == 0xffffffffu;
					}
				}
				if (!valid)
					o = circuit_payload(b->vram, C.psm, addr, 0);
				else
				{
					uint32_t n = C.super_samples / 4;
					uint32_t quad = C.super_samples != 8 ? (y & 1u) + (x & 1u) * 2u : (x & 1u) + (y & 1u) * 2u;
					uint32_t base = 2 + n * quad;
					float v[4] = { 0.0f, 0.0f, 0.0f, 0.0f };
					for (uint32_t i = 0; i < n; i++)
					{
						uint32_t c = circuit_payload(b->vram, C.psm, addr, base + i);
						for (int k = 0; k < 4; k++)
							v[k] = v[k] + oracle::unorm(c, k);
					}
					for (int k = 0; k < 4; k++)
						v[k] = v[k] / float(n);
					o = oracle::pack_unorm(v);
				}
			}
			out[size_t(y) * C.width + x] = o;
		}
	return 0;
}

// ---------------------------------------------------------------------------
// vsync (GSRenderer::vsync, gs/gs_renderer.cpp:4738-5055; extwrite.comp:37-98;
// weave.frag): restated with the definitions the CUDA backend uses for what
// the reference leaves to the rasteriser -- an 8-bit sub-texel bilinear
// stretch clamped to the edge, integer blends rounded to nearest, float
// expressions evaluated left to right with one rounding per operation.

static uint32_t stretch_sample(const std::vector<uint32_t> &img, uint32_t iw, uint32_t ih, int32_t dx, int32_t dy,
                               uint32_t vw, uint32_t vh)
{
	int64_t fx = (int64_t(2 * dx + 1) * iw * 256) / (2 * int64_t(vw)) - 128;
	int64_t fy = (int64_t(2 * dy + 1) * ih * 256) / (2 * int64_t(vh)) - 128;
	int32_t x0 = int32_t(fx >> 8), y0 = int32_t(fy >> 8);
	uint32_t wx = uint32_t(fx & 255), wy = uint32_t(fy & 255);
	auto cl = [](int32_t v, uint32_t n) { return uint32_t(std::min(std::max(v, 0), int32_t(n) - 1)); };
	uint32_t xs[2] = { cl(x0, iw), cl(x0 + 1, iw) }, ys[2] = { cl(y0, ih), cl(y0 + 1, ih) };
	uint32_t wxs[2] = { 256 - wx, wx }, wys[2] = { 256 - wy, wy };
	uint32_t out = 0;
	for (int k = 0; k < 4; k++)
	{
		uint32_t acc = 0;
		for (int j = 0; j < 2; j++)
			for (int i = 0; i < 2; i++)
				acc += wxs[i] * wys[j] * ((img[size_t(ys[j]) * iw + xs[i]] >> (8 * k)) & 255u);
		out |= ((acc + 32768u) >> 16) << (8 * k);
	}
	return out;
}

static uint32_t blend255(uint32_t s, uint32_t d, uint32_t a)
{
	uint32_t v = s * a + d * (255 - a);
	uint32_t q = v / 255, r = v % 255;
	return q + (2 * r > 255 ? 1 : 0);
}

static float luma_diff(uint32_t a, uint32_t b)
{
	float dr = oracle::unorm(a, 0) - oracle::unorm(b, 0);
	float dg = oracle::unorm(a, 1) - oracle::unorm(b, 1);
	float db = oracle::unorm(a, 2) - oracle::unorm(b, 2);
	float s = dr * 0.299f;
	s = s + dg * 0.587f;
	s = s + db * 0.114f;
	return std::fabs(s);
}

static int o_vsync(void *self, const pgs_merge_params *mp, void *dst)
{
	if (!mp || !dst)
		return PGS_ERROR_INVALID_ARGUMENT;
	const pgs_merge_params &M = *mp;
	auto *b = static_cast<Backend *>(self);
	std::vector<uint32_t> circ[2];
	for (int i = 0; i < 2; i++)
	{
		const pgs_circuit_params &c = M.circuit[i];
		if (size_t(c.width) * c.height == 0)
			continue;
		if (c.width > 4096 || c.height > 4096)
			return PGS_ERROR_INVALID_ARGUMENT;
		circ[i].resize(size_t(c.width) * c.height);
		int r = o_circuit(self, &c, circ[i].data());
		if (r)
			return r;
	}
	uint32_t *out = static_cast<uint32_t *>(dst);
	if (M.raw_circuit == 1 || M.raw_circuit == 2)
	{
		const auto &c = circ[M.raw_circuit - 1];
		if (!c.empty())
			memcpy(out, c.data(), c.size() * 4);
		return 0;
	}
	if (M.width == 0 || M.height == 0)
		return 0;
	if (M.width > 4096 || M.height > 4096)
		return PGS_ERROR_INVALID_ARGUMENT;
	if ((M.draw_circuit1 && circ[0].empty()) || (M.draw_circuit2 && circ[1].empty()))
		return PGS_ERROR_INVALID_ARGUMENT;
	const uint32_t W = M.width, H = M.height;
	std::vector<uint32_t> merged(size_t(W) * H);
	auto inside = [&](int i, int32_t x, int32_t y) {
		return M.rect_w[i] && M.rect_h[i] && x >= M.rect_x[i] && x < M.rect_x[i] + int32_t(M.rect_w[i]) &&
		       y >= M.rect_y[i] && y < M.rect_y[i] + int32_t(M.rect_h[i]);
	};
	for (uint32_t y = 0; y < H; y++)
		for (uint32_t x = 0; x < W; x++)
		{
			int32_t ix = int32_t(x), iy = int32_t(y);
			uint32_t color = M.bgcolor & 0xffffffu;
			if (M.draw_circuit2 && inside(1, ix, iy))
				color = stretch_sample(circ[1], M.circuit[1].width, M.circuit[1].height, ix - M.rect_x[1],
				                       iy - M.rect_y[1], M.rect_w[1], M.rect_h[1]);
			if (M.draw_circuit1 && inside(0, ix, iy))
			{
				uint32_t s = stretch_sample(circ[0], M.circuit[0].width, M.circuit[0].height, ix - M.rect_x[0],
				                            iy - M.rect_y[0], M.rect_w[0], M.rect_h[0]);
				if (M.blend == 0)
					color = s;
				else
				{
					uint32_t a = M.blend == 1 ? M.alp : (s >> 24);
					uint32_t o = s & 0xff000000u;
					for (int k = 0; k < 3; k++)
						o |= blend255((s >> (8 * k)) & 255u, (color >> (8 * k)) & 255u, a) << (8 * k);
					color = o;
				}
			}
			merged[size_t(y) * W + x] = color;
		}

	if (M.ext_write && M.ext_width && M.ext_height)
	{
		const std::vector<uint32_t> *src = &merged;
		uint32_t sw = W, sh = H;
		if (M.ext_source == 1 || M.ext_source == 2)
		{
			int ci = M.ext_source == 1 ? 1 : 0;
			if (circ[ci].empty())
				return PGS_ERROR_INVALID_ARGUMENT;
			src = &circ[ci];
			sw = M.circuit[ci].width;
			sh = M.circuit[ci].height;
		}
		if (M.ext_width > 4096 || M.ext_height > 4096)
			return PGS_ERROR_INVALID_ARGUMENT;
		for (uint32_t gy = 0; gy < M.ext_height; gy++)
			for (uint32_t gx = 0; gx < M.ext_width; gx++)
			{
				float u = M.ext_uv_base[0] + float(gx) * M.ext_uv_scale[0];
				float v = M.ext_uv_base[1] + float(gy) * M.ext_uv_scale[1];
				int32_t tx = std::min(std::max(int32_t(std::floor(u * float(sw))), 0), int32_t(sw) - 1);
				int32_t ty = std::min(std::max(int32_t(std::floor(v * float(sh))), 0), int32_t(sh) - 1);
				uint32_t c = (*src)[size_t(ty) * sw + tx];
				float r = oracle::unorm(c, 0), g = oracle::unorm(c, 1), bb = oracle::unorm(c, 2), a = oracle::unorm(c, 3);
				float ey = 0.587f * g;
				ey = ey + 0.114f * bb;
				ey = ey + 0.299f * r;
				float ecb = -0.311f * g;
				ecb = ecb + 0.500f * bb;
				ecb = ecb - 0.169f * r;
				float ecr = -0.419f * g;
				ecr = ecr - 0.081f * bb;
				ecr = ecr + 0.500f * r;
				float Y = (219.0f * ey + 16.0f) / 255.0f;
				float Cb = (224.0f * ecb + 128.0f) / 255.0f;
				float Cr = (224.0f * ecr + 128.0f) / 255.0f;
				float o[4];
				switch (M.ext_emodc)
				{
				case 0: o[0] = r; o[1] = g; o[2] = bb; break;
				case 1: o[0] = Y; o[1] = Y; o[2] = Y; break;
				case 2: o[0] = Y; o[1] = Cb; o[2] = Cr; break;
				default: o[0] = a; o[1] = a; o[2] = a; break;
				}
				switch (M.ext_emoda)
				{
				case 0: o[3] = a; break;
				case 1: o[3] = Y; break;
				case 2: o[3] = 0.5f * Y; break;
				default: o[3] = 0.0f; break;
				}
				uint32_t addr = oracle::swizzle(gx + M.ext_wdx, gy + M.ext_wdy, M.ext_exbp, M.ext_exbw, 0x00);
				uint32_t packed = oracle::pack_unorm(o);
				memcpy(b->vram.data() + size_t(addr) * 4, &packed, 4);
				if (b->num_planes > 1)
					memset(b->vram.data() + oracle::VRAM + size_t(addr) * 4, 0, 4);
			}
	}

	if (!M.deinterlace)
	{
		for (auto &f : b->fields)
			f.clear();
		memcpy(out, merged.data(), merged.size() * 4);
		return 0;
	}
	if (W != b->field_w || H != b->field_h)
	{
		for (auto &f : b->fields)
			f.clear();
		b->field_w = W;
		b->field_h = H;
	}
	for (int i = 3; i >= 1; i--)
		b->fields[i] = std::move(b->fields[i - 1]);
	b->fields[0] = std::move(merged);
	if (b->fields[1].empty())
		b->fields[1] = b->fields[0];
	if (b->fields[2].empty())
		b->fields[2] = b->fields[0];
	if (b->fields[3].empty())
		b->fields[3] = b->fields[1];
	const auto &f0 = b->fields[0], &f1 = b->fields[1], &f2 = b->fields[2], &f3 = b->fields[3];
	const uint32_t H2 = 2 * H;
	for (uint32_t y = 0; y < H2; y++)
		for (uint32_t x = 0; x < W; x++)
		{
			uint32_t o;
			if ((y & 1) == (M.phase & 1))
				o = f0[size_t(y >> 1) * W + x];
			else if (y == 0 || y == H2 - 1)
				o = f1[size_t(y >> 1) * W + x];
			else
			{
				uint32_t up = (y - 1) >> 1;
				uint32_t cur0 = f0[size_t(up) * W + x], cur1 = f0[size_t(up + 1) * W + x];
				uint32_t prev0 = f2[size_t(up) * W + x], prev1 = f2[size_t(up + 1) * W + x];
				uint32_t fld1 = f1[size_t(y >> 1) * W + x], fld3 = f3[size_t(y >> 1) * W + x];
				float mh = luma_diff(cur0, prev0), ml = luma_diff(cur1, prev1), mc = luma_diff(fld1, fld3);
				float diff = std::fmax(std::fmin(mh, ml), mc);
				float tt = (diff - 0.04f) / (0.06f - 0.04f);
				tt = std::fmin(std::fmax(tt, 0.0f), 1.0f);
				float bob = (tt * tt) * (3.0f - 2.0f * tt);
				float c[4];
				for (int k = 0; k < 3; k++)
				{
					float avg = 0.5f * (oracle::unorm(cur0, k) + oracle::unorm(cur1, k));
					c[k] = oracle::unorm(fld1, k) * (1.0f - bob) + avg * bob;
				}
				c[3] = 1.0f;
				o = oracle::pack_unorm(c);
			}
			out[size_t(y) * W + x] = o;
		}
	return 0;
}

static const pgs_backend_ops ORACLE_OPS = {
	PGS_ABI_VERSION, o_destroy, o_reserve, o_flush_rendering, o_copy, o_palette, o_set_ss, o_submit, o_read, o_write, o_error,
	nullptr, nullptr, o_circuit, o_vsync, nullptr, o_snapshot, nullptr,
};

extern "C" {
void *pgs_oracle_backend_create(const pgs_backend_ops **ops)
{
	auto *b = new (std::nothrow) Backend();
	if (ops)
		*ops = &ORACLE_OPS;
	return b;
}

uint64_t pgs_oracle_fragment_count(void *backend)
{
	return static_cast<Backend *>(backend)->fragments.load();
}

// Direct access to the restated swizzle for known-answer tests.
uint32_t pgs_oracle_swizzle(uint32_t x, uint32_t y, uint32_t base, uint32_t stride, uint32_t psm)
{
	return oracle::swizzle(x, y, base, stride, psm);
}

// The phase LUT of the backend's current sampling rate (64 * 64 * 2 + 32 * 32 words).
void pgs_oracle_phase_lut(void *backend, uint32_t *out)
{
	const auto *b = static_cast<const oracle::Backend *>(backend);
	memcpy(out, b->phase_lut, sizeof(b->phase_lut));
}

// Copies up to `max` logged primitive states; returns the number logged.
uint32_t pgs_oracle_state_log(void *backend, uint32_t *out, uint32_t max)
{
	auto &log = static_cast<Backend *>(backend)->state_log;
	for (uint32_t i = 0; i < max && i < log.size(); i++)
		out[i] = log[i];
	return uint32_t(log.size());
}

float pgs_oracle_rcp_fixed(uint32_t b) { return oracle::rcp_fixed(b); }
float pgs_oracle_rcp_float(float v) { return oracle::rcp_float(v); }
}
