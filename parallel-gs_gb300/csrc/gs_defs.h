// gs_defs.h -- constants, register field access and the PS2 swizzle, usable
// from host C++ and from CUDA device code.
//
// Bit positions of the primitive state words follow the reference's shared
// header (gs/shaders/data_structures.h:206-308) because they are part of the
// record format that crosses the frontend/backend boundary.  Register fields
// follow the GS hardware layout (gs/gs_registers.hpp).
#pragma once

#include <stdint.h>

#if defined(__CUDACC__)
#define PGS_HD __host__ __device__ __forceinline__
#else
#define PGS_HD static inline
#endif

namespace pgs
{
// Sub-pixel precision of vertex positions and the raster grid.
constexpr int SUBPIXEL_BITS = 4;
constexpr int SUBPIXELS = 1 << SUBPIXEL_BITS;
constexpr int RASTER_SUBSAMPLE_BITS = 3;
constexpr int RASTER_SUBPIXELS = 1 << RASTER_SUBSAMPLE_BITS;
constexpr int SUBPIXEL_QUANTIZE_BITS = SUBPIXEL_BITS - RASTER_SUBSAMPLE_BITS;
constexpr int SUBPIXELS_RASTER_QUANTIZE = 1 << SUBPIXEL_QUANTIZE_BITS;

constexpr uint32_t BLOCK_BYTES = 256;
constexpr uint32_t PAGE_BYTES = 8192;
constexpr uint32_t BLOCKS_PER_PAGE = 32;
constexpr uint32_t BUFFER_WIDTH_SCALE = 64;
constexpr uint32_t VRAM_SIZE = 4u * 1024u * 1024u;
constexpr uint32_t VRAM_MASK = VRAM_SIZE - 1;

// PrimitiveAttribute::state bits.
constexpr int STATE_BIT_Z_TEST = 12;
constexpr int STATE_BIT_Z_WRITE = 13;
constexpr int STATE_BIT_OPAQUE = 14;
constexpr int STATE_BIT_PARALLELOGRAM = 15;
constexpr int STATE_BIT_MULTISAMPLE = 16;
constexpr int STATE_BIT_Z_TEST_GREATER = 17;
constexpr int STATE_BIT_PERSPECTIVE = 18;
constexpr int STATE_BIT_IIP = 19;
constexpr int STATE_BIT_FIX = 20;
constexpr int STATE_BIT_SPRITE = 21;
constexpr int STATE_BIT_LINE = 22;
constexpr int STATE_BIT_SCANMSK_EVEN = 23;
constexpr int STATE_BIT_SCANMSK_ODD = 24;
constexpr int STATE_BIT_SNAP_RASTER = 25;
constexpr int STATE_BIT_SNAP_ATTRIBUTE = 26;
constexpr int STATE_PARALLELOGRAM_PROVOKING_OFFSET = 27;
constexpr int STATE_VERTEX_RENDER_PASS_INSTANCE_OFFSET = 29;
constexpr uint32_t STATE_INDEX_MASK = 0xfffu;

// PrimitiveAttribute::tex bits.
constexpr uint32_t TEX_TEXTURE_INDEX_MASK = 0xffffu;
constexpr uint32_t TEX_SAMPLER_MAG_LINEAR_BIT = 1u << 16;
constexpr uint32_t TEX_SAMPLER_MIN_LINEAR_BIT = 1u << 17;
constexpr uint32_t TEX_SAMPLER_MIPMAP_LINEAR_BIT = 1u << 18;
constexpr uint32_t TEX_SAMPLER_CLAMP_S_BIT = 1u << 19;
constexpr uint32_t TEX_SAMPLER_CLAMP_T_BIT = 1u << 20;
constexpr int TEX_MAX_MIP_LEVEL_OFFSET = 21;
constexpr uint32_t TEX_PER_SAMPLE_BIT = 1u << 24;
constexpr uint32_t TEX_SAMPLE_MAPPING_BIT = 1u << 25;
constexpr uint32_t TEX_SAMPLE_RESOLVED_BIT = 1u << 26;

// PrimitiveAttribute::tex2 bits.
constexpr uint32_t TEX2_FIXED_LOD_BIT = 1u << 0;

// PrimitiveAttribute::alpha fields.
constexpr int ALPHA_AREF_OFFSET = 0;
constexpr int ALPHA_AFIX_OFFSET = 8;

// StateVector::combiner.
constexpr uint32_t COMBINER_MODE_MASK = 3u;
constexpr uint32_t COMBINER_MODULATE = 0;
constexpr uint32_t COMBINER_DECAL = 1;
constexpr uint32_t COMBINER_HIGHLIGHT = 2;
constexpr uint32_t COMBINER_HIGHLIGHT2 = 3;
constexpr uint32_t COMBINER_TME_BIT = 1u << 2;
constexpr uint32_t COMBINER_FOG_BIT = 1u << 3;
constexpr uint32_t COMBINER_TCC_BIT = 1u << 4;

// StateVector::blend_mode.
constexpr uint32_t BLEND_MODE_ATE_BIT = 1u << 1;
constexpr int BLEND_MODE_ATE_MODE_OFFSET = 2;
constexpr int BLEND_MODE_AFAIL_MODE_OFFSET = 5;
constexpr uint32_t BLEND_MODE_DATE_BIT = 1u << 7;
constexpr uint32_t BLEND_MODE_DATM_BIT = 1u << 8;
constexpr uint32_t BLEND_MODE_ABE_BIT = 1u << 9;
constexpr uint32_t BLEND_MODE_PABE_BIT = 1u << 10;
constexpr int BLEND_MODE_A_MODE_OFFSET = 11;
constexpr int BLEND_MODE_B_MODE_OFFSET = 13;
constexpr int BLEND_MODE_C_MODE_OFFSET = 15;
constexpr int BLEND_MODE_D_MODE_OFFSET = 17;
constexpr uint32_t BLEND_MODE_COLCLAMP_BIT = 1u << 19;
constexpr uint32_t BLEND_MODE_FB_ALPHA_BIT = 1u << 20;
constexpr uint32_t BLEND_MODE_DTHE_BIT = 1u << 21;

// Pixel storage modes.
constexpr uint32_t PSMCT32 = 0x00;
constexpr uint32_t PSMCT24 = 0x01;
constexpr uint32_t PSMCT16 = 0x02;
constexpr uint32_t PSMCT16S = 0x0a;
constexpr uint32_t PSMT8 = 0x13;
constexpr uint32_t PSMT4 = 0x14;
constexpr uint32_t PSMT8H = 0x1b;
constexpr uint32_t PSMT4HL = 0x24;
constexpr uint32_t PSMT4HH = 0x2c;
constexpr uint32_t PSMZ32 = 0x30;
constexpr uint32_t PSMZ24 = 0x31;
constexpr uint32_t PSMZ16 = 0x32;
constexpr uint32_t PSMZ16S = 0x3a;

constexpr uint32_t HOST_TO_LOCAL = 0;
constexpr uint32_t LOCAL_TO_HOST = 1;
constexpr uint32_t LOCAL_TO_LOCAL = 2;

constexpr uint32_t ATST_NEVER = 0, ATST_ALWAYS = 1, ATST_LESS = 2, ATST_LEQUAL = 3,
                   ATST_EQUAL = 4, ATST_GEQUAL = 5, ATST_GREATER = 6, ATST_NOTEQUAL = 7;
constexpr uint32_t AFAIL_KEEP = 0, AFAIL_FB_ONLY = 1, AFAIL_ZB_ONLY = 2, AFAIL_RGB_ONLY = 3;
constexpr uint32_t BLEND_RGB_SOURCE = 0, BLEND_RGB_DEST = 1, BLEND_RGB_ZERO = 2;
constexpr uint32_t BLEND_ALPHA_SOURCE = 0, BLEND_ALPHA_DEST = 1, BLEND_ALPHA_FIX = 2;
constexpr uint32_t WRAP_REPEAT = 0, WRAP_CLAMP = 1, WRAP_REGION_CLAMP = 2, WRAP_REGION_REPEAT = 3;

// 64-bit register field extraction.
PGS_HD uint32_t field(uint64_t reg, int offset, int bits)
{
	return uint32_t((reg >> offset) & ((1ull << bits) - 1ull));
}

PGS_HD uint32_t bits32(uint32_t v, int offset, int count)
{
	return (v >> offset) & ((count == 32) ? 0xffffffffu : ((1u << count) - 1u));
}

PGS_HD bool psm_is_32bit(uint32_t psm) { return psm == PSMCT32 || psm == PSMZ32; }
PGS_HD bool psm_is_24bit(uint32_t psm) { return psm == PSMCT24 || psm == PSMZ24; }
PGS_HD bool psm_is_16bit(uint32_t psm)
{
	return psm == PSMCT16 || psm == PSMCT16S || psm == PSMZ16 || psm == PSMZ16S;
}
PGS_HD bool psm_is_palette(uint32_t psm)
{
	return psm == PSMT8 || psm == PSMT4 || psm == PSMT8H || psm == PSMT4HL || psm == PSMT4HH;
}

PGS_HD uint32_t psm_bits_per_pixel(uint32_t psm)
{
	switch (psm)
	{
	case PSMCT24: case PSMZ24: return 24;
	case PSMCT16: case PSMCT16S: case PSMZ16: case PSMZ16S: return 16;
	case PSMT8: case PSMT8H: return 8;
	case PSMT4: case PSMT4HL: case PSMT4HH: return 4;
	default: return 32;
	}
}

// Page/block geometry per storage format: page is (1<<pw) x (1<<ph) pixels,
// block is (1<<bw) x (1<<bh), a column is (1<<ch) rows.
struct Layout
{
	uint32_t pw, ph, bw, bh, ch;
};

PGS_HD Layout psm_layout(uint32_t psm)
{
	switch (psm)
	{
	case PSMCT16: case PSMCT16S: case PSMZ16: case PSMZ16S: return { 6, 6, 4, 3, 1 };
	case PSMT8: return { 7, 6, 4, 4, 2 };
	case PSMT4: return { 7, 7, 5, 4, 2 };
	default: return { 6, 5, 3, 3, 1 };
	}
}

// Block index inside a page for the 32-bit family: bits x2 y1 x1 y0 x0.
PGS_HD uint32_t block_order_32(uint32_t bx, uint32_t by)
{
	return (bx & 1u) | ((by & 1u) << 1) | ((bx & 2u) << 1) | ((by & 2u) << 2) | ((bx & 4u) << 2);
}

// Block index for the 16-bit family and PSMT4: bits y2 x1 y1 x0 y0.
PGS_HD uint32_t block_order_16(uint32_t bx, uint32_t by)
{
	return (by & 1u) | ((bx & 1u) << 1) | ((by & 2u) << 1) | ((bx & 2u) << 2) | ((by & 4u) << 2);
}

// Block index for PSMCT16S: bits x1 y1 y2 x0 y0.
PGS_HD uint32_t block_order_16s(uint32_t bx, uint32_t by)
{
	return (by & 1u) | ((bx & 1u) << 1) | (by & 4u) | ((by & 2u) << 2) | ((bx & 2u) << 3);
}

// GS local memory address of pixel (x, y) for a buffer at base_block (256-byte
// units) with row stride page_stride (64-pixel units).  Units of the result:
// 32-bit words for 32/24-bit formats, 16-bit halves for 16-bit formats, bytes
// for PSMT8, nibbles for PSMT4 (the reference's swizzle_PS2,
// gs/shaders/swizzle_utils.h:329-522).
PGS_HD uint32_t swizzle_address(uint32_t x, uint32_t y, uint32_t base_block, uint32_t page_stride, uint32_t psm)
{
	Layout L = psm_layout(psm);
	if (psm == PSMT4 || psm == PSMT8)
		page_stride >>= 1;
	uint32_t page = (y >> L.ph) * page_stride + (x >> L.pw);
	uint32_t bx = (x & ((1u << L.pw) - 1u)) >> L.bw;
	uint32_t by = (y & ((1u << L.ph) - 1u)) >> L.bh;
	uint32_t column = (y & ((1u << L.bh) - 1u)) >> L.ch;
	uint32_t px = x & ((1u << L.bw) - 1u);
	uint32_t py = y & ((1u << L.ch) - 1u);
	uint32_t column_base;

	switch (psm)
	{
	case PSMZ32: case PSMZ24:
	{
		uint32_t block = (block_order_32(bx, by) + base_block) ^ 0x18u;
		uint32_t pix = (px & 1u) | ((py & 1u) << 1) | ((px & 2u) << 1) | ((px & 4u) << 1);
		column_base = page * PAGE_BYTES + block * BLOCK_BYTES + column * 64u;
		return ((column_base + pix * 4u) & VRAM_MASK) >> 2;
	}
	case PSMCT16: case PSMZ16: case PSMCT16S: case PSMZ16S:
	{
		uint32_t block;
		if (psm == PSMCT16 || psm == PSMZ16)
			block = block_order_16(bx, by) + base_block;
		else
			block = block_order_16s(bx, by) + base_block;
		if (psm == PSMZ16 || psm == PSMZ16S)
			block ^= 0x18u;
		uint32_t pix = ((px & 8u) >> 3) | ((px & 1u) << 1) | ((py & 1u) << 2) | ((px & 2u) << 2) | ((px & 4u) << 2);
		column_base = page * PAGE_BYTES + block * BLOCK_BYTES + column * 64u;
		return ((column_base + pix * 2u) & VRAM_MASK) >> 1;
	}
	case PSMT8:
	{
		uint32_t block = block_order_32(bx, by) + base_block;
		uint32_t pix = ((py & 2u) >> 1) | ((px & 8u) >> 2) | ((px & 1u) << 2) | ((py & 1u) << 3) |
		               ((px & 2u) << 3) | ((((px & 4u) << 3) ^ ((py & 2u) << 4)) ^ ((column & 1u) << 5));
		column_base = page * PAGE_BYTES + block * BLOCK_BYTES + column * 64u;
		return (column_base + pix) & VRAM_MASK;
	}
	case PSMT4:
	{
		uint32_t block = block_order_16(bx, by) + base_block;
		uint32_t pix = ((py & 2u) >> 1) | ((px & 8u) >> 2) | ((px & 16u) >> 2) | ((px & 1u) << 3) |
		               ((py & 1u) << 4) | ((px & 2u) << 4) |
		               ((((px & 4u) << 4) ^ ((py & 2u) << 5)) ^ ((column & 1u) << 6));
		column_base = page * PAGE_BYTES + block * BLOCK_BYTES + column * 64u;
		return ((column_base << 1) + pix) & ((VRAM_MASK << 1) | 1u);
	}
	default:
	{
		uint32_t block = block_order_32(bx, by) + base_block;
		uint32_t pix = (px & 1u) | ((py & 1u) << 1) | ((px & 2u) << 1) | ((px & 4u) << 1);
		column_base = page * PAGE_BYTES + block * BLOCK_BYTES + column * 64u;
		return ((column_base + pix * 4u) & VRAM_MASK) >> 2;
	}
	}
}

// RGBA5551 -> RGBA8888 with TEXA alpha expansion (utils.h:79-87).
PGS_HD uint32_t rgba16_to_rgba32(uint32_t c16, uint32_t aem, uint32_t ta0, uint32_t ta1)
{
	uint32_t r = (c16 & 0x1fu) << 3;
	uint32_t g = ((c16 >> 5) & 0x1fu) << 3;
	uint32_t b = ((c16 >> 10) & 0x1fu) << 3;
	uint32_t a_bit = (c16 >> 15) & 1u;
	uint32_t a = (aem && c16 == 0) ? 0u : (a_bit ? ta1 : ta0);
	return r | (g << 8) | (b << 16) | ((a & 0xffu) << 24);
}

PGS_HD uint32_t rgba32_to_rgba16(uint32_t c)
{
	return ((c >> 3) & 0x1fu) | (((c >> 11) & 0x1fu) << 5) | (((c >> 19) & 0x1fu) << 10) | (((c >> 31) & 1u) << 15);
}

PGS_HD uint32_t rgb24_to_rgba32(uint32_t c, uint32_t aem, uint32_t ta0)
{
	uint32_t rgb = c & 0xffffffu;
	uint32_t a = (aem && rgb == 0) ? 0u : ta0;
	return rgb | ((a & 0xffu) << 24);
}
} // namespace pgs
