// ref_harness.cpp -- TEST INFRASTRUCTURE ONLY.
// Compiles the reference's own CPU swizzle path (gs/gs_util.hpp:49-205,
// vram_readback/vram_upload over swizzle_PS2 from gs/shaders/swizzle_utils.h)
// from the sources where they lie, with a shim for the absent Granite headers,
// and exports it through a C ABI.  Used to pin the oracle's and the CUDA
// backend's VRAM layout, and as the timed reference CPU baseline for
// swizzled uploads and readbacks.
#include <stdio.h>
#define LOGW(...) fprintf(stderr, __VA_ARGS__)
#include "gs_util.hpp"

using namespace ParallelGS;

extern "C" {
uint32_t pgs_ref_swizzle(uint32_t x, uint32_t y, uint32_t base, uint32_t stride, uint32_t psm, uint32_t vram_mask)
{
	return swizzle_PS2(x, y, base, stride, psm, vram_mask);
}

int pgs_ref_vram_upload(uint32_t psm, void *vram, const void *data, uint32_t base, uint32_t stride,
                        uint32_t x, uint32_t y, uint32_t w, uint32_t h, uint32_t vram_mask)
{
	switch (psm)
	{
#define D(p) case p: vram_upload<p>(vram, data, base, stride, x, y, w, h, vram_mask); return 0
	D(PSMCT32); D(PSMCT24); D(PSMCT16); D(PSMCT16S); D(PSMZ32); D(PSMZ24); D(PSMZ16); D(PSMZ16S);
	D(PSMT8); D(PSMT8H); D(PSMT4); D(PSMT4HL); D(PSMT4HH);
#undef D
	default: return -1;
	}
}

int pgs_ref_vram_readback(uint32_t psm, void *out, const void *vram, uint32_t base, uint32_t stride,
                          uint32_t x, uint32_t y, uint32_t w, uint32_t h, uint32_t vram_mask)
{
	switch (psm)
	{
#define D(p) case p: vram_readback<p>(out, vram, base, stride, x, y, w, h, vram_mask); return 0
	D(PSMCT32); D(PSMCT24); D(PSMCT16); D(PSMCT16S); D(PSMZ32); D(PSMZ24); D(PSMZ16); D(PSMZ16S);
	D(PSMT8); D(PSMT8H);
#undef D
	default: return -1;
	}
}
}
