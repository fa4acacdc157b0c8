// frontend.cpp -- GSInterface re-hosted without Vulkan (gs/gs_interface.cpp).
//
// The frontend ingests GIF packets and register writes, keeps the GS register
// file and the 3-entry vertex queue, turns drawing kicks into primitive records
// (pgs_vertex_position / pgs_vertex_attribute / pgs_primitive_attribute),
// batches them into render passes and drives a backend through
// pgs_backend_ops.  Primitive records follow drawing_kick_append
// (gs/gs_interface.cpp:2473-2836); state words follow drawing_kick_update_state
// (:1804-1968) and drawing_kick_update_state_vector (:1065-1128).
//
// Triangle pairs that tile a rectangle are fused into parallelograms as
// gs/gs_util.cpp:237-377 decides.  Differences from the reference, all
// result-neutral for sequential GS semantics: no palette memoization
// (:689-799), no feedback-texture modes (:2140-2330) and a page-granular hazard
// tracker.  Because the backend samples textures straight from VRAM instead of
// from snapshot images, the tracker also ends a render pass when a transfer or
// a framebuffer write would touch pages an earlier primitive of the same pass
// samples.
#include "pgs.h"
#include "gs_defs.h"
#include "gs_tracker.h"

#include <algorithm>
#include <atomic>
#include <condition_variable>
#include <cstddef>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <memory>
#include <mutex>
#include <new>
#include <thread>
#include <unistd.h>
#include <unordered_map>
#include <vector>

using namespace pgs;

namespace
{
// A+D register addresses (gs/gs_register_addr.hpp).
enum Reg : uint32_t
{
	R_PRIM = 0x00, R_RGBAQ = 0x01, R_ST = 0x02, R_UV = 0x03, R_XYZF2 = 0x04, R_XYZ2 = 0x05,
	R_TEX0_1 = 0x06, R_TEX0_2 = 0x07, R_CLAMP_1 = 0x08, R_CLAMP_2 = 0x09, R_FOG = 0x0a,
	R_XYZF3 = 0x0c, R_XYZ3 = 0x0d, R_RGBAQ_UNDOC = 0x11, R_TEX1_1 = 0x14, R_TEX1_2 = 0x15,
	R_TEX2_1 = 0x16, R_TEX2_2 = 0x17, R_XYOFFSET_1 = 0x18, R_XYOFFSET_2 = 0x19,
	R_PRMODECONT = 0x1a, R_PRMODE = 0x1b, R_TEXCLUT = 0x1c, R_SCANMSK = 0x22,
	R_MIPTBP1_1 = 0x34, R_MIPTBP1_2 = 0x35, R_MIPTBP2_1 = 0x36, R_MIPTBP2_2 = 0x37,
	R_TEXA = 0x3b, R_FOGCOL = 0x3d, R_TEXFLUSH = 0x3f, R_SCISSOR_1 = 0x40, R_SCISSOR_2 = 0x41,
	R_ALPHA_1 = 0x42, R_ALPHA_2 = 0x43, R_DIMX = 0x44, R_DTHE = 0x45, R_COLCLAMP = 0x46,
	R_TEST_1 = 0x47, R_TEST_2 = 0x48, R_PABE = 0x49, R_FBA_1 = 0x4a, R_FBA_2 = 0x4b,
	R_FRAME_1 = 0x4c, R_FRAME_2 = 0x4d, R_ZBUF_1 = 0x4e, R_ZBUF_2 = 0x4f,
	R_BITBLTBUF = 0x50, R_TRXPOS = 0x51, R_TRXREG = 0x52, R_TRXDIR = 0x53, R_HWREG = 0x54,
	R_SIGNAL = 0x60, R_FINISH = 0x61, R_LABEL = 0x62
};

// FlushReason, numbered as the reference's (gs/page_tracker.hpp:117-126).
enum FlushReason : uint32_t
{
	FLUSH_FB_POINTER = PGS_FLUSH_FB_POINTER, FLUSH_OVERFLOW = PGS_FLUSH_OVERFLOW,
	FLUSH_TEXTURE_HAZARD = PGS_FLUSH_TEXTURE_HAZARD, FLUSH_COPY_HAZARD = PGS_FLUSH_COPY_HAZARD,
	FLUSH_EXPLICIT = PGS_FLUSH_SUBMISSION, FLUSH_PRESSURE = PGS_FLUSH_PRESSURE, FLUSH_HOST_ACCESS = PGS_FLUSH_HOST_ACCESS
};

enum PrimType : uint32_t
{
	PRIM_POINT = 0, PRIM_LINE_LIST = 1, PRIM_LINE_STRIP = 2, PRIM_TRI_LIST = 3,
	PRIM_TRI_STRIP = 4, PRIM_TRI_FAN = 5, PRIM_SPRITE = 6, PRIM_INVALID = 7
};

constexpr uint32_t NUM_PAGES = VRAM_SIZE / PAGE_BYTES;

// Register views.  Field offsets are those of the GS hardware registers.
struct PrimReg
{
	uint32_t prim, iip, tme, fge, abe, aa1, fst, ctxt, fix;
	explicit PrimReg(uint64_t r)
	    : prim(field(r, 0, 3)), iip(field(r, 3, 1)), tme(field(r, 4, 1)), fge(field(r, 5, 1)),
	      abe(field(r, 6, 1)), aa1(field(r, 7, 1)), fst(field(r, 8, 1)), ctxt(field(r, 9, 1)),
	      fix(field(r, 10, 1)) {}
	bool enables_aa1() const { return aa1 && prim != PRIM_SPRITE && prim != PRIM_POINT; }
};

struct Tex0Reg
{
	uint32_t tbp0, tbw, psm, tw, th, tcc, tfx, cbp, cpsm, csm, csa, cld;
	explicit Tex0Reg(uint64_t r)
	    : tbp0(field(r, 0, 14)), tbw(field(r, 14, 6)), psm(field(r, 20, 6)), tw(field(r, 26, 4)),
	      th(field(r, 30, 4)), tcc(field(r, 34, 1)), tfx(field(r, 35, 2)), cbp(field(r, 37, 14)),
	      cpsm(field(r, 51, 4)), csm(field(r, 55, 1)), csa(field(r, 56, 5)), cld(field(r, 61, 3)) {}
};

struct TestReg
{
	uint32_t ate, atst, aref, afail, date, datm, zte, ztst;
	explicit TestReg(uint64_t r)
	    : ate(field(r, 0, 1)), atst(field(r, 1, 3)), aref(field(r, 4, 8)), afail(field(r, 12, 2)),
	      date(field(r, 14, 1)), datm(field(r, 15, 1)), zte(field(r, 16, 1)), ztst(field(r, 17, 2)) {}
	bool has_z_test() const { return ztst > 1; }
};

struct AlphaReg
{
	uint32_t a, b, c, d, fix;
	explicit AlphaReg(uint64_t r)
	    : a(field(r, 0, 2)), b(field(r, 2, 2)), c(field(r, 4, 2)), d(field(r, 6, 2)), fix(field(r, 32, 8)) {}
};

struct FrameReg
{
	uint32_t fbp, fbw, psm, fbmsk;
	explicit FrameReg(uint64_t r)
	    : fbp(field(r, 0, 9)), fbw(field(r, 16, 6)), psm(field(r, 24, 6)), fbmsk(field(r, 32, 32)) {}
};

struct ZbufReg
{
	uint32_t zbp, psm, zmsk;
	explicit ZbufReg(uint64_t r) : zbp(field(r, 0, 9)), psm(field(r, 24, 4)), zmsk(field(r, 32, 1)) {}
};

struct ClampReg
{
	uint32_t wms, wmt, minu, maxu, minv, maxv;
	explicit ClampReg(uint64_t r)
	    : wms(field(r, 0, 2)), wmt(field(r, 2, 2)), minu(field(r, 4, 10)), maxu(field(r, 14, 10)),
	      minv(field(r, 24, 10)), maxv(field(r, 34, 10)) {}
};

struct Tex1Reg
{
	uint32_t lcm, mxl, mmag, mmin, mtba, l, k;
	explicit Tex1Reg(uint64_t r)
	    : lcm(field(r, 0, 1)), mxl(field(r, 2, 3)), mmag(field(r, 5, 1)), mmin(field(r, 6, 3)),
	      mtba(field(r, 9, 1)), l(field(r, 19, 2)), k(field(r, 32, 12)) {}
	bool mmin_has_mipmap() const { return mmin > 1 && mmin <= 5; }
};

// Two 64-bit lanes (GCC/Clang vector extension, lowered to SSE on x86-64 and
// NEON on AArch64).
typedef uint64_t Word2 __attribute__((vector_size(16), aligned(4), may_alias));

// Records ahead of the one being written whose arena lines are prefetched.
static constexpr uint32_t ARENA_PREFETCH_RECORDS = 12;

// A write prefetch of the line `offset` bytes past `base` (which may lie past
// the end of the buffer: a prefetch never faults).
static inline void prefetch_for_write(const void *base, size_t offset)
{
	__builtin_prefetch(reinterpret_cast<const void *>(reinterpret_cast<uintptr_t>(base) + offset), 1, 3);
}

// Vertex copy in the widths the vertex queue writes: the 16-byte position,
// then the attributes as 16 + 8 bytes.
static __attribute__((always_inline)) inline void copy_vertex(pgs_vertex_position &dp, pgs_vertex_attribute &da, const pgs_vertex_position &sp,
                               const pgs_vertex_attribute &sa)
{
	static_assert(sizeof(pgs_vertex_position) == 16 && sizeof(pgs_vertex_attribute) == 24, "vertex layout");
	Word2 p, lo;
	uint64_t hi;
	memcpy(&p, &sp, 16);
	memcpy(&lo, &sa, 16);
	memcpy(&hi, reinterpret_cast<const char *>(&sa) + 16, 8);
	memcpy(&dp, &p, 16);
	memcpy(&da, &lo, 16);
	memcpy(reinterpret_cast<char *>(&da) + 16, &hi, 8);
}

static bool frame_compat(uint64_t a, uint64_t b)
{
	// FBP, FBW, PSM must match; FBMSK may differ (FRAMEBits::compat).
	return (a & 0x3f3f01ffull) == (b & 0x3f3f01ffull);
}

static bool zbuf_compat(uint64_t a, uint64_t b)
{
	return (a & 0x0f0001ffull) == (b & 0x0f0001ffull);
}

struct Instance
{
	int32_t bb[4] = { INT32_MAX, INT32_MAX, INT32_MIN, INT32_MIN };
	uint64_t frame = 0, zbuf = 0;
	uint32_t color_write_mask = 0;
	uint32_t fb_pw = 0, fb_ph = 0, z_pw = 0, z_ph = 0;
	bool z_sensitive = false, z_write = false;
	bool has_channel_shuffle = false, z_feedback = false;
};

// Dirty state (StateDirtyFlags, gs/gs_interface.hpp:116-129): which derived
// state a register write may have changed.  Register writes set bits only
// when the value changes; a committed primitive clears them all.
enum DirtyBits : uint32_t
{
	DIRTY_DEGENERATE = 1u << 0, DIRTY_PRIM_TEMPLATE = 1u << 1, DIRTY_TEX = 1u << 2, DIRTY_FB = 1u << 3,
	DIRTY_FEEDBACK = 1u << 4, DIRTY_SCISSOR = 1u << 5, DIRTY_STATE = 1u << 6, DIRTY_POTENTIAL_FEEDBACK_REGION = 1u << 7,
	DIRTY_ALL = 0xffu
};

// How a textured draw relates to the framebuffer it writes
// (FBFeedbackMode, gs/gs_interface.hpp).
enum FeedbackMode : uint32_t
{
	FEEDBACK_NONE, FEEDBACK_PIXEL, FEEDBACK_SLICED, FEEDBACK_BYPASS_HAZARDS
};

// The render pass's texture feedback kind (RenderPass::Feedback).
enum PassFeedback : uint32_t
{
	PASS_FEEDBACK_NONE, PASS_FEEDBACK_COLOR, PASS_FEEDBACK_DEPTH
};

struct TextureKey
{
	pgs_texture_desc d;
	bool operator==(const TextureKey &o) const { return memcmp(&d, &o.d, sizeof(d)) == 0; }
};

struct TextureKeyHash
{
	size_t operator()(const TextureKey &k) const
	{
		const uint32_t *w = reinterpret_cast<const uint32_t *>(&k.d);
		uint64_t h = 1469598103934665603ull;
		for (size_t i = 0; i < sizeof(k.d) / 4; i++)
			h = (h ^ w[i]) * 1099511628211ull;
		return size_t(h);
	}
};
} // namespace

struct pgs_gs : TrackerClient
{
	const pgs_backend_ops *ops = nullptr;
	void *be = nullptr;

	uint64_t regs[128] = {};
	// Privileged registers PMODE .. BGCOLOR (gs/gs_interface.hpp:70-91).
	uint64_t priv[15] = {};
	// GS dump being replayed / recorded.
	FILE *dump_in = nullptr, *dump_out = nullptr;
	std::vector<uint64_t> dump_buf;
	uint32_t cached_cbp[2] = {};

	struct Path
	{
		uint64_t tag_lo = 0, tag_hi = 0;
		uint32_t nloop = 0, flg = 0, nreg = 0;
		uint32_t reg = 0, loop = 0;
	};

	// Vertex assembly state: GIF paths, the vertex registers (RGBAQ, ST, UV,
	// FOG, the internal Q), the vertex queue and its own copies of the
	// registers vertex assembly reads (PRIM as drawn, PRMODECONT, XYOFFSET).
	// Only the decoder touches it while a transfer runs, so the decoder can
	// run on a thread of its own ahead of the register-file state; regs[]
	// gets the vertex registers back when the transfer ends.  On a cache line
	// of its own: the state thread never shares one with it.
	struct alignas(64) Decoder
	{
		Path paths[4];
		uint64_t rgbaq = 0, st = 0, uv = 0, fog = 0;
		float internal_q = 1.0f;
		uint64_t prim = 0, prmodecont = 0, xyoffset[2] = {};
		int32_t ofx = 0, ofy = 0;
		// Vertex queue.  A vertex is written as one 16-byte position word and
		// a 16 + 8 byte attribute pair and read back with the same widths, so
		// the reads forward from the stores still in flight.
		struct
		{
			pgs_vertex_position pos[3];
			pgs_vertex_attribute attr[3];
			uint32_t count = 0;
		} vq;
	} dec;

	// Render pass under construction.
	pgs_vertex_position *positions = nullptr;
	pgs_vertex_attribute *attributes = nullptr;
	pgs_primitive_attribute *prims = nullptr;
	uint32_t primitive_count = 0;
	std::vector<pgs_state_vector> state_vectors;
	std::vector<pgs_texture_desc> textures;
	Instance instances[PGS_MAX_RENDER_PASS_INSTANCES];
	uint32_t num_instances = 1;
	uint32_t current_instance = 0;
	bool has_aa1 = false, has_scanmsk = false, has_mipmap = false, has_ss_textures = false;
	bool ssaa_textures = false; // super_sampled_textures of set_super_sampling_rate
	// Field-aware rendering, chosen by the last vsync (gs/gs_interface.cpp:4662-4672):
	// high-resolution read-out of field-rendered interlaced output.
	bool field_aware = false;
	// Hacks (gs/gs_interface.hpp:209-237).
	bool hack_disable_mipmaps = false, hack_unsynced_readbacks = false, hack_blend_demote = false;
	// Vsyncs left with progressive read-out switched off after a tall
	// SCANMSK primitive (gs/gs_interface.cpp:1947-1959, 4631-4637).
	uint32_t complex_scanmsk_timeout = 0;
	pgs_signal_interface signal_iface = {};
	// Triangle-pair fusion (gs/gs_interface.cpp:2569-2602): the last committed
	// triangle could be the first half of a rectangle, its vertex order, and
	// the transfer count when it was drawn.
	bool last_para_candidate = false;
	uint32_t last_para_order[3] = { 0, 1, 2 };
	pgs_debug_mode debug_mode = {};
	uint32_t clut_instance = 0;
	uint32_t pending_palette_updates = 0;
	// CLUT ring numbering of the reference's renderer (update_palette_cache,
	// rewind_clut_instance, gs/gs_renderer.cpp:3364-3419): the newest slot,
	// whether a texture read it since it was written, and the loads not yet
	// flushed to the cache (format bits and the slot each started from).
	uint32_t ring_next = 0, latest_clut_instance = 0;
	bool ring_last_read = false;
	struct RingLoad
	{
		uint32_t cpsm, csa;
		bool is8;
		uint32_t incoming;
	};
	std::vector<RingLoad> ring_pending;
	// Palette loads of the pass that can be reused by an identical load
	// (memoized_palettes, gs/gs_interface.cpp:685-799): a sliding window.
	struct MemoizedPalette
	{
		uint32_t instance, csa_mask;
		uint64_t tex0, texclut;
		uint32_t incoming;
	};
	MemoizedPalette memo[16];
	uint32_t num_memo = 0;

	// Cached primitive template; recomputed when template_dirty is set.
	bool template_dirty = true;
	uint32_t tpl_state = 0, tpl_tex = 0, tpl_tex2 = 0;
	// Pages of every sampled mip level of the current template's texture.

	// Caches of values derived from the register file.  reg_serial changes
	// whenever a register other than vertex data (RGBAQ, ST, UV, FOG, XYZ*) is
	// written or the sampling rate changes; fb_epoch whenever the render pass
	// is flushed.
	uint64_t reg_serial = 1, fb_epoch = 1, tpl_serial = 1;
	uint64_t degenerate_serial = 0;
	bool degenerate_cached = false;
	uint64_t fb_state_serial = 0, fb_state_epoch = 0;
	struct DrawConsts
	{
		uint64_t serial = 0;
		int32_t snap = 0;
		int32_t sci_lo[2] = {}, sci_hi[2] = {};
		int32_t sci_hi_x_fb = 0;
		bool can_wrap = false, line_aa1 = false, tme = false, z_sens = false;
		FrameReg frame{ 0 };
		ZbufReg zb{ 0 };
		uint32_t alpha_word = 0, fogcol = 0;
		// Page geometry of the colour and depth buffers (page_span).
		uint32_t fb_pw = 0, fb_ph = 0, fb_stride = 0, z_pw = 0, z_ph = 0, z_stride = 0;
	} dc;

	// Marks every value derived from the register file dirty after the file
	// was replaced wholesale (clobber_register_state).
	void clobber_state()
	{
		reg_serial++;
		template_dirty = true;
		dirty = DIRTY_ALL;
		decoder_load();
	}

	// The decoder's copies from the register file, after the file was set
	// from outside a transfer (reset, dump restore, clobber).
	void decoder_load()
	{
		dec.rgbaq = regs[R_RGBAQ];
		dec.st = regs[R_ST];
		dec.uv = regs[R_UV];
		dec.fog = regs[R_FOG];
		dec.prim = regs[R_PRIM];
		dec.prmodecont = regs[R_PRMODECONT];
		dec.xyoffset[0] = regs[R_XYOFFSET_1];
		dec.xyoffset[1] = regs[R_XYOFFSET_2];
		dec.vq.count = 0;
		update_offsets();
	}

	// Register file reads and side-effect free writes from the host: the
	// vertex registers live in the decoder while a transfer runs (a host
	// callback may ask), and the decoder's copies follow direct writes.
	uint64_t read_reg(uint32_t addr) const
	{
		switch (addr)
		{
		case R_RGBAQ: return dec.rgbaq;
		case R_ST: return dec.st;
		case R_UV: return dec.uv;
		case R_FOG: return dec.fog;
		default: return regs[addr];
		}
	}

	void set_reg(uint32_t addr, uint64_t v)
	{
		regs[addr] = v;
		switch (addr)
		{
		case R_RGBAQ: dec.rgbaq = v; break;
		case R_ST: dec.st = v; break;
		case R_UV: dec.uv = v; break;
		case R_FOG: dec.fog = v; break;
		case R_PRIM: dec.prim = v; break;
		case R_PRMODECONT: dec.prmodecont = v; break;
		case R_XYOFFSET_1: case R_XYOFFSET_2: dec.xyoffset[addr - R_XYOFFSET_1] = v; break;
		default: break;
		}
	}

	// The vertex registers back into the register file (read_register, dumps).
	void decoder_store()
	{
		regs[R_RGBAQ] = dec.rgbaq;
		regs[R_ST] = dec.st;
		regs[R_UV] = dec.uv;
		regs[R_FOG] = dec.fog;
	}

	void record_transfer(uint32_t path, const void *data, size_t size)
	{
		uint8_t type = 0, p = uint8_t(path);
		uint32_t sz = uint32_t(size);
		if (fwrite(&type, 1, 1, dump_out) != 1 || fwrite(&p, 1, 1, dump_out) != 1 ||
		    fwrite(&sz, 4, 1, dump_out) != 1 || fwrite(data, 1, size, dump_out) != size)
		{
			fclose(dump_out);
			dump_out = nullptr;
			sticky_error = PGS_ERROR_IO;
		}
	}

	const DrawConsts &draw_consts()
	{
		if (dc.serial == reg_serial)
			return dc;
		PrimReg prim(regs[R_PRIM]);
		// Field-aware rendering keeps the untightened box
		// (gs/gs_interface.cpp:2528-2531).
		dc.snap = field_aware ? 0 : (1 << int(SUBPIXEL_BITS - sampling_rate_y_log2)) - 1;
		uint64_t sc = ctx_reg(R_SCISSOR_1);
		dc.frame = FrameReg(ctx_reg(R_FRAME_1));
		dc.zb = ZbufReg(ctx_reg(R_ZBUF_1));
		dc.sci_lo[0] = int32_t(field(sc, 0, 11));
		dc.sci_lo[1] = int32_t(field(sc, 32, 11));
		dc.sci_hi[0] = int32_t(field(sc, 16, 11));
		dc.sci_hi[1] = int32_t(field(sc, 48, 11));
		int32_t fb_width = int32_t(std::max<uint32_t>(1, dc.frame.fbw) * BUFFER_WIDTH_SCALE);
		dc.sci_hi_x_fb = std::min(dc.sci_hi[0], fb_width - 1);
		dc.can_wrap = dc.frame.fbw != 0 && dc.sci_hi_x_fb < dc.sci_hi[0];
		dc.line_aa1 = prim.enables_aa1();
		dc.tme = prim.tme != 0;
		dc.z_sens = state_is_z_sensitive();
		AlphaReg alpha(ctx_reg(R_ALPHA_1));
		TestReg test(ctx_reg(R_TEST_1));
		dc.alpha_word = (alpha.fix << ALPHA_AFIX_OFFSET) | (test.aref << ALPHA_AREF_OFFSET);
		dc.fogcol = uint32_t(regs[R_FOGCOL]);
		uint32_t row = dc.frame.fbw ? dc.frame.fbw : 1;
		Layout FL = psm_layout(dc.frame.psm), ZL = psm_layout(dc.zb.psm | 0x30);
		dc.fb_pw = FL.pw;
		dc.fb_ph = FL.ph;
		dc.fb_stride = (dc.frame.psm == PSMT4 || dc.frame.psm == PSMT8) ? row >> 1 : row;
		dc.z_pw = ZL.pw;
		dc.z_ph = ZL.ph;
		dc.z_stride = row;
		dc.serial = reg_serial;
		return dc;
	}

	HazardTracker tracker{ *this };

	// Drawing state of the reference's state tracker (gs/gs_interface.hpp:386-430).
	uint32_t dirty = DIRTY_ALL;
	uint64_t texflush_counter = 0;
	bool texflush_pending = false;
	uint32_t last_texture_index = UINT32_MAX;
	uint64_t last_texture_valid_at = 0;
	pgs_texture_desc last_texture_desc = {};
	// Page rectangles of each level of the current texture state.
	PageRect tex_rects[7];
	uint32_t tex_num_rects = 0;
	// The pass's texture table by descriptor hash (TextureStateToLocalIndex).
	struct TexEntry
	{
		uint32_t index;
		uint64_t valid_at;
		bool long_term, valid;
	};
	std::unordered_map<uint64_t, TexEntry> tex_entries;
	// Texture feedback against the current frame / depth buffer
	// (update_color_feedback_state, gs/gs_interface.cpp:2141-2308).
	bool is_color_feedback = false, is_depth_feedback = false, is_awkward_color_feedback = false;
	bool is_potential_feedback = false, is_potential_channel_shuffle = false, current_is_channel_shuffle = false;
	struct
	{
		uint32_t base_page, pw, ph, page_stride, width_bias, max_safe_page;
	} potential = {};
	uint32_t pass_feedback = PASS_FEEDBACK_NONE, pass_feedback_psm = 0, pass_feedback_cpsm = 0;
	bool has_hazardous_short_term = false, has_optimized_short_term = false;
	// Work submitted since the last submission; its limits end a pass early
	// (check_flush_stats, gs/gs_renderer.cpp:864-895).
	struct
	{
		uint64_t prims, passes, copies, palettes, copy_threads, scratch;
	} pending = {};
	// Blocks of each page that textures of the open pass read.  The backend
	// decodes those textures as the pass begins, so a transfer into them has
	// to end the pass first.
	uint32_t pass_tex_blocks[NUM_PAGES] = {};
	std::vector<uint16_t> pass_tex_pages;
	// VRAM snapshots of the open pass and the texture count at each.
	uint32_t num_snapshots = 0;
	uint32_t snapshot_textures[PGS_MAX_VRAM_SNAPSHOTS] = {};

	struct
	{
		std::vector<uint64_t> payload;
		bool active = false;
		uint32_t required_qwords = 0;
		uint32_t flushed_qwords = 0;
		uint64_t bitbltbuf = 0, trxpos = 0, trxreg = 0, trxdir = 0;
		std::vector<uint8_t> fifo;
		uint32_t fifo_offset = 0, fifo_size = 0;
	} xfer;

	uint32_t sampling_rate_x_log2 = 0, sampling_rate_y_log2 = 0;
	pgs_flush_stats stats = {};
	int sticky_error = 0;

	// ---------------------------------------------------------------
	uint64_t ctx_reg(uint32_t base_addr) const
	{
		return regs[base_addr + field(regs[R_PRIM], 9, 1)];
	}

	void reserve_buffers()
	{
		int r = ops->reserve_primitive_buffers(be, PGS_MAX_PRIMITIVES_PER_FLUSH, &positions, &attributes, &prims);
		if (r != 0)
			sticky_error = r;
	}

	static void rates_for(uint32_t ss, bool ordered, uint32_t &x, uint32_t &y)
	{
		switch (ss)
		{
		case 2: x = 0; y = 1; break;
		case 4:
			if (ordered) { x = 1; y = 1; }
			else { x = 0; y = 2; }
			break;
		case 8: x = 1; y = 2; break;
		case 16:
			if (ordered) { x = 2; y = 2; }
			else { x = 1; y = 3; }
			break;
		default: x = 0; y = 0; break;
		}
	}

	// GSInterface::set_super_sampling_rate (gs/gs_interface.cpp:64-117): the
	// rate is lowered to the most the backend supports (the reference takes
	// min(requested, get_max_supported_super_sampling())); this backend table
	// has no such query, so the rate steps down by halves until the backend
	// accepts it.  At 1x super-sampled textures are off.
	void set_super_sampling(uint32_t ss, bool ordered, bool ss_textures)
	{
		if (ss != 2 && ss != 4 && ss != 8 && ss != 16)
			ss = 1;
		int r = 0;
		for (;;)
		{
			rates_for(ss, ordered, sampling_rate_x_log2, sampling_rate_y_log2);
			r = ops->set_super_sampling(be, sampling_rate_x_log2, sampling_rate_y_log2);
			if (r != PGS_ERROR_UNSUPPORTED || ss == 1)
				break;
			ss >>= 1;
		}
		ssaa_textures = ss_textures && ss > 1;
		reg_serial++;
		template_dirty = true;
		if (r != 0)
			sticky_error = r;
	}

	// ---------------------------------------------------------------
	// Flushes go through the tracker, which clears its per-pass marks and
	// calls back (PageTracker::flush_render_pass, gs/page_tracker.cpp:497-509).
	void flush_render_pass(uint32_t reason) { tracker.flush_render_pass(reason); }

	// GSInterface::flush(flags, reason) (gs/gs_interface.cpp:353-420).
	void tracker_flush(uint32_t flags, uint32_t reason) override
	{
		if (flags & TRACKER_FLUSH_CACHE)
		{
			// flush_cache_upload: pending CLUT loads reach the ring, and
			// memoised palettes are forgotten (gs/gs_interface.cpp:386-393).
			tracker.clear_cache_pages();
			ring_pending.clear();
			num_memo = 0;
		}
		if (flags & TRACKER_FLUSH_FB)
			do_flush_render_pass(reason);
		if (reason == FLUSH_PRESSURE)
		{
			tracker.mark_submission(FLUSH_EXPLICIT);
			submit();
		}
	}

	void tracker_invalidate_texture(uint64_t hash, bool clut) override
	{
		if (!clut)
		{
			auto it = tex_entries.find(hash);
			if (it != tex_entries.end())
				it->second.valid = false;
		}
		mark_texture_state_dirty();
	}

	void tracker_texture_state_dirty_with_flush() override
	{
		mark_texture_state_dirty();
		texflush_counter++;
	}

	void tracker_forget_memoization() override
	{
		num_memo = 0;
		mark_texture_state_dirty();
	}

	void mark_texture_state_dirty()
	{
		last_texture_index = UINT32_MAX;
		last_texture_valid_at = 0;
		dirty |= DIRTY_PRIM_TEMPLATE | DIRTY_TEX;
	}

	void submit()
	{
		int r = ops->flush_submit(be);
		if (r != 0)
			sticky_error = r;
		pending = {};
	}

	// Limits of pending work (gs/gs_renderer.cpp:31-39, 864-895): past any of
	// them the next draw kick or TEX0 write ends the open pass.
	void check_pending_work()
	{
		if (pending.prims >= 4096 || pending.passes >= 1024 || pending.scratch >= 100ull * 1000 * 1000 ||
		    pending.copies >= 16 * 1024 || pending.palettes >= 4096)
			tracker.mark_memory_pressure();
	}

	void mark_pass_texture(const PageRect &r)
	{
		for (uint32_t y = 0; y < r.page_height; y++)
			for (uint32_t x = 0; x < r.page_width; x++)
			{
				uint32_t p = (r.base_page + y * r.page_stride + x) & (NUM_PAGES - 1);
				if (!pass_tex_blocks[p])
					pass_tex_pages.push_back(uint16_t(p));
				pass_tex_blocks[p] |= r.block_mask;
			}
	}

	// A transfer or host write is about to replace blocks that textures of
	// the open pass read.  The reference samples those textures from cache
	// images taken before (flush_cached); here the textures held so far decode
	// from a VRAM snapshot taken now, or the pass ends where the backend keeps
	// no snapshots.
	void protect_pass_textures(const PageRect &r, uint32_t reason)
	{
		if (!pass_texture_hit(r))
			return;
		if (ops->abi_version >= 5 && ops->snapshot_vram && num_snapshots < PGS_MAX_VRAM_SNAPSHOTS)
		{
			int slot = ops->snapshot_vram(be);
			if (slot >= 0)
			{
				snapshot_textures[num_snapshots++] = uint32_t(textures.size());
				for (uint16_t p : pass_tex_pages)
					pass_tex_blocks[p] = 0;
				pass_tex_pages.clear();
				return;
			}
			if (slot != PGS_ERROR_CAPACITY)
			{
				sticky_error = slot;
				return;
			}
		}
		flush_render_pass(reason);
	}

	bool pass_texture_hit(const PageRect &r) const
	{
		if (pass_tex_pages.empty())
			return false;
		for (uint32_t y = 0; y < r.page_height; y++)
			for (uint32_t x = 0; x < r.page_width; x++)
				if (pass_tex_blocks[(r.base_page + y * r.page_stride + x) & (NUM_PAGES - 1)] & r.block_mask)
					return true;
		return false;
	}

	// ---------------------------------------------------------------
	// Render pass flush (gs/gs_interface.cpp:133-351).
	void do_flush_render_pass(uint32_t reason)
	{
		fb_epoch++;
		last_para_candidate = false;
		if (primitive_count)
		{
			pgs_render_pass rp = {};
			rp.positions = positions;
			rp.attributes = attributes;
			rp.prims = prims;
			rp.num_primitives = primitive_count;
			rp.states = state_vectors.data();
			rp.num_states = uint32_t(state_vectors.size());
			rp.textures = textures.data();
			rp.num_textures = uint32_t(textures.size());
			rp.flush_reason = reason;
			rp.has_aa1 = has_aa1;
			rp.has_scanmsk = has_scanmsk;
			rp.has_mipmap = has_mipmap;
			rp.has_ss_textures = has_ss_textures;
			rp.field_aware = field_aware;
			rp.blend_demote = hack_blend_demote;
			rp.num_snapshots = num_snapshots;
			memcpy(rp.snapshot_textures, snapshot_textures, sizeof(snapshot_textures));

			uint64_t binning_cost = 0;
			for (uint32_t i = 0; i < num_instances; i++)
			{
				auto &inst = instances[i];
				if (inst.bb[2] < 0)
					continue;
				uint64_t tw = uint64_t((inst.bb[2] - inst.bb[0]) >> 3) + 1;
				uint64_t th = uint64_t((inst.bb[3] - inst.bb[1]) >> 3) + 1;
				binning_cost += tw * th * primitive_count;
			}

			uint32_t ts;
			if (binning_cost < 10ull * 1000)
				ts = 3;
			else if (binning_cost < 10ull * 1000 * 1000)
				ts = 4;
			else if (binning_cost < 100ull * 1000 * 1000)
				ts = 5;
			else
				ts = 6;
			if (sampling_rate_y_log2 != 0 && ts > 3)
				ts -= 1;

			for (uint32_t i = 0; i < num_instances; i++)
			{
				auto &inst = instances[i];
				if (inst.bb[2] < 0)
					continue;
				uint64_t cw = uint64_t((inst.bb[2] - inst.bb[0]) >> ts) + 1;
				uint64_t ch = uint64_t((inst.bb[3] - inst.bb[1]) >> ts) + 1;
				uint64_t list_size = cw * ch * primitive_count * sizeof(uint16_t);
				while (list_size > 48ull * 1024 * 1024)
				{
					ts += 1;
					list_size /= 4;
				}
			}
			rp.coarse_tile_size_log2 = ts;

			uint32_t n = num_instances;
			if (instances[n - 1].bb[2] < 0)
				n--;
			rp.num_instances = n;

			for (uint32_t i = 0; i < n; i++)
			{
				auto &inst = instances[i];
				auto &pass = rp.instances[i];
				pass.frame = inst.frame;
				pass.zbuf = inst.zbuf;
				pass.base_x = inst.bb[0];
				pass.base_y = inst.bb[1];
				pass.coarse_tiles_width = uint32_t((inst.bb[2] - inst.bb[0]) >> ts) + 1;
				pass.coarse_tiles_height = uint32_t((inst.bb[3] - inst.bb[1]) >> ts) + 1;
				pass.sampling_rate_x_log2 = sampling_rate_x_log2;
				pass.sampling_rate_y_log2 = sampling_rate_y_log2;
				pass.opaque_fbmask = ~inst.color_write_mask;

				FrameReg frame(inst.frame);
				ZbufReg zbuf(inst.zbuf);
				bool channel_shuffle = inst.has_channel_shuffle;
				if (frame.psm != PSMCT32 && frame.psm != PSMCT24 && frame.psm != PSMZ32 && frame.psm != PSMZ24)
				{
					uint32_t m = inst.color_write_mask & 0xf8f8f8u;
					channel_shuffle = channel_shuffle || (m != 0xf8f8f8u && m != 0);
				}
				pass.channel_shuffle = channel_shuffle;

				// Field-aware rendering, or super-sampled textures in the
				// pass, keep the pass super-sampled; channel shuffles, depth
				// feedback and frame/depth aliasing with depth writes do not
				// (gs/gs_interface.cpp:225-260).
				if ((sampling_rate_x_log2 | sampling_rate_y_log2) != 0 && !field_aware && !(ssaa_textures && has_ss_textures))
				{
					if (channel_shuffle || inst.z_feedback || (inst.z_write && zbuf.zbp == frame.fbp))
					{
						pass.sampling_rate_x_log2 = 0;
						pass.sampling_rate_y_log2 = 0;
					}
				}
				pass.z_sensitive = inst.z_sensitive;
				pass.z_write = inst.z_write;
			}

			int r = ops->flush_rendering(be, &rp);
			if (r != 0)
				sticky_error = r;
			stats.num_render_passes++;
			stats.num_primitives += primitive_count;
			stats.num_flushes_by_reason[reason & 7]++;
			pending.prims += primitive_count;
			pending.passes += rp.num_instances;
			check_pending_work();
		}
		else if (num_snapshots)
		{
			// Release the snapshot slots of a pass that drew nothing.
			pgs_render_pass empty = {};
			int r = ops->flush_rendering(be, &empty);
			if (r != 0)
				sticky_error = r;
		}
		num_snapshots = 0;

		Instance keep = instances[current_instance];
		for (auto &inst : instances)
			inst = Instance();
		instances[0].frame = keep.frame;
		instances[0].zbuf = keep.zbuf;
		instances[0].fb_pw = keep.fb_pw;
		instances[0].fb_ph = keep.fb_ph;
		instances[0].z_pw = keep.z_pw;
		instances[0].z_ph = keep.z_ph;
		num_instances = 1;
		current_instance = 0;
		primitive_count = 0;
		state_vectors.clear();
		textures.clear();
		tex_entries.clear();
		pending_palette_updates = 0;
		has_aa1 = false;
		has_scanmsk = false;
		has_mipmap = false;
		has_ss_textures = false;
		last_para_candidate = false;
		pass_feedback = PASS_FEEDBACK_NONE;
		has_hazardous_short_term = false;
		has_optimized_short_term = false;
		template_dirty = true;
		dirty = DIRTY_ALL;
		for (uint16_t p : pass_tex_pages)
			pass_tex_blocks[p] = 0;
		pass_tex_pages.clear();
		// A pass that ended on an older memoised palette rewinds the ring
		// (rewind_clut_instance, gs/gs_renderer.cpp:3384-3398).
		if (clut_instance != ring_next)
		{
			tracker.register_clut_read(PageRect(), 0xffffffffu);
			tracker.invalidate_texture_cache(clut_instance);
		}
		ring_next = clut_instance;
		latest_clut_instance = clut_instance;
		reserve_buffers();
	}

	// GSInterface::flush (gs/gs_interface.cpp:4257-4264).
	void flush()
	{
		flush_pending_transfer(true);
		tracker.mark_submission(FLUSH_EXPLICIT);
		submit();
	}

	// ---------------------------------------------------------------
	// Transfers (gs/gs_interface.cpp:2979-3276).
	void init_transfer()
	{
		flush_pending_transfer(false);
		xfer.bitbltbuf = regs[R_BITBLTBUF];
		xfer.trxpos = regs[R_TRXPOS];
		xfer.trxreg = regs[R_TRXREG];
		xfer.trxdir = regs[R_TRXDIR];
		uint32_t xdir = field(xfer.trxdir, 0, 2);
		uint32_t rrw = field(xfer.trxreg, 0, 12), rrh = field(xfer.trxreg, 32, 12);
		uint32_t dbp = field(xfer.bitbltbuf, 32, 14), dbw = field(xfer.bitbltbuf, 48, 6), dpsm = field(xfer.bitbltbuf, 56, 6);
		uint32_t sbp = field(xfer.bitbltbuf, 0, 14), sbw = field(xfer.bitbltbuf, 16, 6), spsm = field(xfer.bitbltbuf, 24, 6);
		uint32_t dsax = field(xfer.trxpos, 32, 11), dsay = field(xfer.trxpos, 48, 11);
		uint32_t ssax = field(xfer.trxpos, 0, 11), ssay = field(xfer.trxpos, 16, 11);

		if (xdir == LOCAL_TO_LOCAL)
		{
			// init_transfer (gs/gs_interface.cpp:3168-3202).
			const PageRect dst = compute_page_rect(dbp, dsax, dsay, rrw, rrh, dbw, dpsm);
			const PageRect src = compute_page_rect(sbp, ssax, ssay, rrw, rrh, sbw, spsm);
			tracker.mark_transfer_copy(dst, src);
			tracker.invalidate_texture_cache(clut_instance);
			protect_pass_textures(dst, FLUSH_COPY_HAZARD);
			pending.copies++;
			pending.copy_threads += uint64_t(rrw) * rrh;
			check_pending_work();
			pgs_copy_desc d = {};
			d.bitbltbuf = xfer.bitbltbuf;
			d.trxpos = xfer.trxpos;
			d.trxreg = xfer.trxreg;
			d.trxdir = xfer.trxdir;
			int r = ops->copy_vram(be, &d);
			if (r != 0)
				sticky_error = r;
			stats.num_copies++;
			template_dirty = true;
		}
		else if (xdir == HOST_TO_LOCAL)
		{
			xfer.required_qwords = uint32_t((uint64_t(rrw) * rrh * psm_bits_per_pixel(dpsm)) / 64);
			xfer.active = xfer.required_qwords != 0;
			xfer.payload.clear();
			xfer.flushed_qwords = 0;
		}
		else if (xdir == LOCAL_TO_HOST)
		{
			// Unsubmitted writes to the source: submit first (init_transfer,
			// gs/gs_interface.cpp:3214-3245).
			const PageRect src = compute_page_rect(sbp, ssax, ssay, rrw, rrh, sbw, spsm);
			if (tracker.host_read_pending(src))
			{
				tracker.mark_submission(FLUSH_HOST_ACCESS);
				submit();
			}
			uint32_t bytes = uint32_t((uint64_t(rrw) * rrh * psm_bits_per_pixel(spsm)) / 8);
			xfer.fifo.assign((bytes + 15) & ~15u, 0);
			xfer.fifo_offset = 0;
			xfer.fifo_size = bytes / 16;
			readback_to_fifo(sbp, sbw, spsm, ssax, ssay, rrw, rrh);
		}
	}

	void readback_to_fifo(uint32_t sbp, uint32_t sbw, uint32_t spsm, uint32_t sx, uint32_t sy, uint32_t w, uint32_t h)
	{
		if (ops->abi_version >= 6 && ops->readback_rect)
		{
			// The backend de-swizzles the rectangle itself.
			pgs_copy_desc d = {};
			d.bitbltbuf = xfer.bitbltbuf;
			d.trxpos = xfer.trxpos;
			d.trxreg = xfer.trxreg;
			d.trxdir = xfer.trxdir;
			int r = ops->readback_rect(be, &d, xfer.fifo.data(), xfer.fifo.size());
			if (r != 0)
				sticky_error = r;
			return;
		}
		std::vector<uint8_t> vram(VRAM_SIZE);
		int r = ops->read_vram(be, 0, 0, VRAM_SIZE, vram.data());
		if (r != 0)
		{
			sticky_error = r;
			return;
		}
		// LOCAL->HOST de-swizzle (vram_readback, gs/gs_util.hpp:50-110).
		uint8_t *dst = xfer.fifo.data();
		for (uint32_t y = 0; y < h; y++)
		{
			uint32_t ey = (y + sy) & 2047;
			for (uint32_t x = 0; x < w; x++)
			{
				uint32_t ex = (x + sx) & 2047;
				uint32_t i = y * w + x;
				uint32_t a = swizzle_address(ex, ey, sbp, sbw, spsm);
				switch (spsm)
				{
				case PSMCT32: case PSMZ32: memcpy(dst + 4 * i, &vram[4 * a], 4); break;
				case PSMCT24: case PSMZ24: memcpy(dst + 3 * i, &vram[4 * a], 3); break;
				case PSMCT16: case PSMCT16S: case PSMZ16: case PSMZ16S: memcpy(dst + 2 * i, &vram[2 * a], 2); break;
				case PSMT8: dst[i] = vram[a]; break;
				case PSMT8H: dst[i] = vram[4 * a + 3]; break;
				default: break;
				}
			}
		}
	}

	void flush_pending_transfer(bool keep_alive)
	{
		if (xfer.active && xfer.payload.size() > xfer.flushed_qwords)
		{
			uint32_t rrw = field(xfer.trxreg, 0, 12), rrh = field(xfer.trxreg, 32, 12);
			uint32_t dbp = field(xfer.bitbltbuf, 32, 14), dbw = field(xfer.bitbltbuf, 48, 6), dpsm = field(xfer.bitbltbuf, 56, 6);
			uint32_t dsax = field(xfer.trxpos, 32, 11), dsay = field(xfer.trxpos, 48, 11);
			// flush_pending_transfer (gs/gs_interface.cpp:2979-3148): a whole
			// single-page upload with no unsubmitted GPU work on its page is
			// written by the host at once, otherwise it is a tracked transfer.
			const PageRect dst = compute_page_rect(dbp, dsax, dsay, rrw, rrh, dbw, dpsm);
			const uint64_t have = uint64_t(xfer.payload.size()), from = xfer.flushed_qwords;
			const bool host_copy = dst.page_width == 1 && dst.page_height == 1 && from == 0 &&
			                       have == xfer.required_qwords && !tracker.host_write_pending(dst);
			if (host_copy)
				tracker.commit_host_write(dst);
			else
				tracker.mark_transfer_write(dst);
			protect_pass_textures(dst, FLUSH_COPY_HAZARD);
			pending.copies++;
			pending.copy_threads += uint64_t(rrw) * rrh;
			if (!host_copy)
				pending.scratch += have * sizeof(uint64_t);
			check_pending_work();

			pgs_copy_desc d = {};
			d.bitbltbuf = xfer.bitbltbuf;
			d.trxpos = xfer.trxpos;
			d.trxreg = xfer.trxreg;
			d.trxdir = xfer.trxdir;
			d.host_data = xfer.payload.data();
			d.host_size = xfer.payload.size() * sizeof(uint64_t);
			d.host_offset = uint64_t(xfer.flushed_qwords) * sizeof(uint64_t);
			d.host_required = uint64_t(xfer.required_qwords) * sizeof(uint64_t);
			int r = ops->copy_vram(be, &d);
			if (r != 0)
				sticky_error = r;
			stats.num_copies++;
			xfer.flushed_qwords = uint32_t(xfer.payload.size());
			template_dirty = true;
			tracker.invalidate_texture_cache(clut_instance);
		}

		if (!keep_alive)
		{
			xfer.payload.clear();
			xfer.flushed_qwords = 0;
			xfer.active = false;
		}
	}

	void hwreg(const uint64_t *data, size_t count)
	{
		if (!xfer.active)
			return;
		xfer.payload.insert(xfer.payload.end(), data, data + count);
		if (xfer.payload.size() >= xfer.required_qwords)
			flush_pending_transfer(false);
	}

	// ---------------------------------------------------------------
	// CLUT loads (handle_clut_upload, gs/gs_interface.cpp:550-799).
	void handle_clut_upload(uint32_t ctx)
	{
		Tex0Reg t(regs[R_TEX0_1 + ctx]);
		uint32_t cpsm = t.cpsm == PSMCT24 ? PSMCT32 : t.cpsm;
		if (!psm_is_palette(t.psm))
			return;

		bool load = false;
		switch (t.cld)
		{
		case 1: load = true; break;
		case 2: case 3: load = true; cached_cbp[t.cld & 1] = t.cbp; break;
		case 4: case 5:
			load = cached_cbp[t.cld & 1] != t.cbp;
			cached_cbp[t.cld & 1] = t.cbp;
			break;
		default: break;
		}
		if (!load)
			return;

		if (xfer.active && xfer.payload.size() > xfer.flushed_qwords)
			flush_pending_transfer(true);

		uint32_t csa = t.csa;
		if (cpsm == PSMCT32)
			csa &= 15;

		uint32_t pw, ph;
		bool is8 = t.psm == PSMT8 || t.psm == PSMT8H;
		if (is8)
		{
			pw = t.csm ? 256 : 16;
			ph = t.csm ? 1 : 16;
		}
		else
		{
			// The reference's page rectangle for a 4-bit CLUT in rectangle
			// layout is 8 x 4 (gs/gs_interface.cpp:624-635).
			pw = t.csm ? 16 : 8;
			ph = t.csm ? 1 : 4;
		}

		uint64_t texclut = regs[R_TEXCLUT];
		uint32_t cbw = field(texclut, 0, 6), cou = field(texclut, 6, 6), cov = field(texclut, 12, 10);
		uint32_t xo = t.csm ? cou * 16 : 0, yo = t.csm ? cov : 0;
		// The CLUT source is read like a texture, and its cached copy goes
		// stale with the CSA banks it fills (handle_clut_upload,
		// gs/gs_interface.cpp:620-683).
		const PageRect src = compute_page_rect(t.cbp, xo, yo, pw, ph, cbw, cpsm);
		uint32_t csa_mask = is8 ? (0xffffu << csa) : (1u << csa);
		if (cpsm == PSMCT32)
			csa_mask |= csa_mask << 16;
		tracker.mark_texture_read(src);
		tracker.register_clut_read(src, csa_mask);

		// Normalise TEX0 to the fields that affect the palette load.
		uint64_t tex0 = regs[R_TEX0_1 + ctx];
		uint64_t keep = (0x3full << 20) | (0x3fffull << 37) | (0x1ull << 55);
		tex0 &= keep;
		tex0 |= uint64_t(cpsm) << 51;
		tex0 |= uint64_t(csa) << 56;

		pgs_palette_upload u = {};
		u.tex0 = tex0;
		u.texclut = texclut;
		u.csm2_x_scale = 1.0f;
		u.csm2_x_bias = 0;
		u.base_instance = clut_instance;

		// An identical load earlier in the pass is reused, unless a later
		// partial load changed banks it did not write (gs/gs_interface.cpp:685-729).
		uint32_t punchthrough = UINT32_MAX;
		for (uint32_t i = num_memo; i; i--)
		{
			const MemoizedPalette &m = memo[i - 1];
			if (m.csa_mask & ~csa_mask)
			{
				if (punchthrough != UINT32_MAX || m.csa_mask != UINT32_MAX)
					break;
				punchthrough = m.instance;
				continue;
			}
			if (m.csa_mask == csa_mask && m.tex0 == u.tex0 && m.texclut == u.texclut)
			{
				if (punchthrough != UINT32_MAX && punchthrough != m.incoming)
					break;
				if (m.instance != clut_instance)
					mark_texture_state_dirty();
				clut_instance = m.instance;
				if (i < num_memo)
				{
					MemoizedPalette moved = m;
					memmove(memo + i - 1, memo + i, (num_memo - i) * sizeof(memo[0]));
					moved.csa_mask = csa_mask;
					moved.tex0 = u.tex0;
					moved.texclut = u.texclut;
					moved.incoming = u.base_instance;
					memo[num_memo - 1] = moved;
				}
				return;
			}
		}

		// A load nothing has read yet is rewritten in place by one that
		// replaces it (same CPSM, CSA and index width), starting from the
		// same palette (update_palette_cache, gs/gs_renderer.cpp:3400-3419).
		const bool numbered = ops->abi_version >= 5;
		const bool replace = numbered && !ring_last_read && !ring_pending.empty() &&
		                     ring_pending.back().cpsm == cpsm && ring_pending.back().csa == csa &&
		                     ring_pending.back().is8 == is8;
		uint32_t incoming = clut_instance;
		if (replace)
			u.base_instance = ring_pending.back().incoming;
		else
		{
			ring_next = (ring_next + 1) % PGS_CLUT_INSTANCES;
			ring_pending.push_back({ cpsm, csa, is8, clut_instance });
			pending.palettes++;
		}
		ring_last_read = false;
		if (numbered)
			u.target = ring_next + 1;
		int inst = ops->update_palette_cache(be, &u);
		if (inst < 0)
		{
			sticky_error = inst;
			return;
		}
		if (!numbered)
			ring_next = uint32_t(inst);
		clut_instance = uint32_t(inst);
		template_dirty = true;
		stats.num_palette_updates++;
		check_pending_work();
		const bool replacing = latest_clut_instance == clut_instance;
		latest_clut_instance = clut_instance;
		mark_texture_state_dirty();
		if (replacing)
		{
			// The replaced load's memo entry goes; the new one keeps its start.
			for (uint32_t i = 0; i < num_memo; i++)
				if (memo[i].instance == clut_instance)
				{
					incoming = memo[i].incoming;
					num_memo--;
					memmove(memo + i, memo + i + 1, (num_memo - i) * sizeof(memo[0]));
					break;
				}
		}
		if (num_memo == 16)
		{
			memmove(memo, memo + 1, 15 * sizeof(memo[0]));
			num_memo--;
		}
		memo[num_memo++] = { clut_instance, csa_mask, u.tex0, u.texclut, incoming };
		if (!replacing)
		{
			pending_palette_updates++;
			if (pending_palette_updates >= PGS_CLUT_INSTANCES)
				flush_render_pass(FLUSH_OVERFLOW);
		}
	}

	void handle_miptbl_gen(uint32_t ctx)
	{
		Tex1Reg tex1(regs[R_TEX1_1 + ctx]);
		if (!tex1.mtba)
			return;
		Tex0Reg t(regs[R_TEX0_1 + ctx]);
		uint32_t base = t.tbp0;
		uint32_t w = 1u << t.tw, h = 1u << t.th;
		uint32_t row = w / 64;
		Layout L = psm_layout(t.psm);
		uint32_t nblocks = (w >> L.bw) * (h >> L.bh);
		base += nblocks;
		nblocks /= 4;
		row /= 2;
		uint64_t m = 0;
		m |= uint64_t(base & 0x3fff) | (uint64_t(row & 0x3f) << 14);
		base += nblocks;
		nblocks /= 4;
		row /= 2;
		m |= (uint64_t(base & 0x3fff) << 20) | (uint64_t(row & 0x3f) << 34);
		base += nblocks;
		m |= (uint64_t(base & 0x3fff) << 40) | (uint64_t(row & 0x3f) << 54);
		regs[R_MIPTBP1_1 + ctx] = m;
		template_dirty = true;
		dirty |= DIRTY_TEX | DIRTY_PRIM_TEMPLATE;
	}

	// ---------------------------------------------------------------
	// Register writes (the a_d_* handlers, gs/gs_interface.cpp:3506-3990):
	// each register marks the derived state it feeds dirty when its value
	// changes (update_internal_register).
	void set_state_reg(uint32_t addr, uint64_t v, uint32_t flags)
	{
		if (regs[addr] != v)
		{
			regs[addr] = v;
			dirty |= flags;
		}
	}

	void set_prim_reg(uint64_t v)
	{
		// PRIM with PRMODECONT.AC = 1, or PRMODE's attributes with the current
		// primitive type (a_d_PRIM / a_d_PRMODE).
		if (field(regs[R_PRIM], 9, 1) != field(v, 9, 1))
			dirty |= DIRTY_DEGENERATE | DIRTY_PRIM_TEMPLATE | DIRTY_TEX | DIRTY_FB | DIRTY_FEEDBACK | DIRTY_SCISSOR;
		set_state_reg(R_PRIM, v, DIRTY_FEEDBACK | DIRTY_PRIM_TEMPLATE | DIRTY_TEX | DIRTY_STATE);
		if (!field(regs[R_PRIM], 4, 1))
			dirty &= ~DIRTY_TEX;
	}

	// A register write on the register-file side: every register except the
	// vertex registers and vertex kicks, which vertex assembly handles
	// (assemble_register) before passing the rest on in stream order.
	void write_state_register(uint32_t addr, uint64_t v)
	{
		addr &= 0x7f;
		switch (addr)
		{
		case R_RGBAQ: case R_RGBAQ_UNDOC: case R_ST: case R_UV: case R_FOG:
		case R_XYZF2: case R_XYZ2: case R_XYZF3: case R_XYZ3:
		case R_BITBLTBUF: case R_TRXPOS: case R_TRXREG: case R_TRXDIR: case R_HWREG:
		case R_SIGNAL: case R_FINISH: case R_LABEL:
			break;
		default:
			reg_serial++;
			break;
		}
		switch (addr)
		{
		case R_PRIM:
		{
			if (field(regs[R_PRMODECONT], 0, 1))
				set_prim_reg(v);
			else
			{
				if ((regs[R_PRIM] & 7ull) != (v & 7ull) && field(v, 7, 1))
					dirty |= DIRTY_PRIM_TEMPLATE;
				regs[R_PRIM] = (regs[R_PRIM] & ~7ull) | (v & 7ull);
			}
			template_dirty = true;
			break;
		}
		case R_PRMODE:
			if (!field(regs[R_PRMODECONT], 0, 1))
			{
				set_prim_reg((v & ~7ull) | (regs[R_PRIM] & 7ull));
				template_dirty = true;
			}
			break;
		case R_TEX0_1: case R_TEX0_2:
			// a_d_TEX0 + handle_tex0_write (gs/gs_interface.cpp:802-805).
			set_state_reg(addr, v, DIRTY_FEEDBACK | DIRTY_STATE | DIRTY_PRIM_TEMPLATE | DIRTY_TEX);
			template_dirty = true;
			handle_clut_upload(addr - R_TEX0_1);
			tracker.flush_if_memory_pressure();
			handle_miptbl_gen(addr - R_TEX0_1);
			break;
		case R_TEX2_1: case R_TEX2_2:
		{
			// TEX2 writes PSM and CLUT fields of TEX0 only (a_d_TEX2, :2950-2968).
			uint32_t ctx = addr - R_TEX2_1;
			uint64_t preserve_mask = 0x3fffull | (0x3full << 14) | (0xfull << 26) | (0xfull << 30) |
			                         (1ull << 34) | (3ull << 35);
			uint64_t t = (regs[R_TEX0_1 + ctx] & preserve_mask) | (v & ~preserve_mask);
			write_state_register(R_TEX0_1 + ctx, t);
			break;
		}
		case R_CLAMP_1: case R_CLAMP_2: case R_TEX1_1: case R_TEX1_2:
			set_state_reg(addr, v, DIRTY_FEEDBACK | DIRTY_PRIM_TEMPLATE | DIRTY_TEX);
			template_dirty = true;
			break;
		case R_SCANMSK:
			set_state_reg(addr, v, DIRTY_PRIM_TEMPLATE);
			template_dirty = true;
			break;
		case R_MIPTBP1_1: case R_MIPTBP1_2: case R_MIPTBP2_1: case R_MIPTBP2_2: case R_TEXA:
			set_state_reg(addr, v, DIRTY_PRIM_TEMPLATE | DIRTY_TEX);
			template_dirty = true;
			break;
		case R_SCISSOR_1: case R_SCISSOR_2:
			set_state_reg(addr, v, DIRTY_SCISSOR | DIRTY_DEGENERATE);
			template_dirty = true;
			break;
		case R_ALPHA_1: case R_ALPHA_2:
			set_state_reg(addr, v, DIRTY_STATE | DIRTY_PRIM_TEMPLATE | DIRTY_DEGENERATE);
			template_dirty = true;
			break;
		case R_DIMX: case R_DTHE: case R_COLCLAMP: case R_PABE: case R_FBA_1: case R_FBA_2:
			set_state_reg(addr, v, DIRTY_STATE | DIRTY_PRIM_TEMPLATE);
			template_dirty = true;
			break;
		case R_TEST_1: case R_TEST_2:
			set_state_reg(addr, v, DIRTY_DEGENERATE | DIRTY_STATE | DIRTY_PRIM_TEMPLATE);
			template_dirty = true;
			break;
		case R_FRAME_1: case R_FRAME_2:
			set_state_reg(addr, v, DIRTY_DEGENERATE | DIRTY_FEEDBACK | DIRTY_TEX | DIRTY_FB | DIRTY_PRIM_TEMPLATE |
			                           DIRTY_SCISSOR);
			template_dirty = true;
			break;
		case R_ZBUF_1: case R_ZBUF_2:
			set_state_reg(addr, v, DIRTY_FEEDBACK | DIRTY_DEGENERATE | DIRTY_TEX | DIRTY_FB | DIRTY_PRIM_TEMPLATE);
			template_dirty = true;
			break;
		case R_XYOFFSET_1: case R_XYOFFSET_2:
			regs[addr] = v;
			break;
		case R_TEXFLUSH:
			// Counted only when a held texture is next used (a_d_TEXFLUSH,
			// gs/gs_interface.cpp:3778-3793).
			texflush_pending = true;
			break;
		case R_BITBLTBUF: case R_TRXPOS: case R_TRXREG:
			regs[addr] = v;
			break;
		case R_TRXDIR:
			regs[addr] = v;
			init_transfer();
			break;
		case R_HWREG:
			hwreg(&v, 1);
			break;
		case R_SIGNAL: case R_FINISH: case R_LABEL:
		{
			// a_d_SIGNAL / FINISH / LABEL (gs/gs_interface.cpp:3970-3988).
			pgs_signal_fn fn = addr == R_SIGNAL ? signal_iface.on_signal :
			                   addr == R_FINISH ? signal_iface.on_finish : signal_iface.on_label;
			if (fn && fn(signal_iface.user, v))
				flush();
			break;
		}
		default:
			// PRMODECONT, TEXCLUT, FOGCOL and the rest: stored, no derived state.
			regs[addr] = v;
			break;
		}
	}

	void update_offsets()
	{
		uint64_t xy = dec.xyoffset[field(dec.prim, 9, 1)];
		dec.ofx = int32_t(field(xy, 0, 16));
		dec.ofy = int32_t(field(xy, 32, 16));
	}

	// ---------------------------------------------------------------
	// Vertex queue (gs/gs_interface.cpp:843-897).
	__attribute__((always_inline)) inline void shift_queue()
	{
		auto &vq = dec.vq;
		if (vq.count == 3)
		{
			copy_vertex(vq.pos[0], vq.attr[0], vq.pos[1], vq.attr[1]);
			copy_vertex(vq.pos[1], vq.attr[1], vq.pos[2], vq.attr[2]);
			vq.count = 2;
		}
	}

	// The queue entry: position (x, y, z, 0) and attributes (s, t, q, rgba |
	// fog, u, v) packed into words in registers and stored whole.
	__attribute__((always_inline)) inline void push_vertex(uint64_t v, uint32_t z, float fog)
	{
		shift_queue();
		auto &vq = dec.vq;
		const uint64_t st = dec.st, rgbaq = dec.rgbaq, uv = dec.uv;
		const uint32_t x = uint32_t(int32_t(field(v, 0, 16)) - dec.ofx);
		const uint32_t y = uint32_t(int32_t(field(v, 16, 16)) - dec.ofy);
		uint32_t fog_bits;
		memcpy(&fog_bits, &fog, 4);
		const Word2 pos = { uint64_t(x) | (uint64_t(y) << 32), uint64_t(z) };
		const Word2 lo = { st, (rgbaq >> 32) | (rgbaq << 32) };
		const uint64_t hi = uint64_t(fog_bits) | (uint64_t(field(uv, 0, 14)) << 32) | (uint64_t(field(uv, 16, 14)) << 48);
		memcpy(&vq.pos[vq.count], &pos, 16);
		memcpy(&vq.attr[vq.count], &lo, 16);
		memcpy(reinterpret_cast<char *>(&vq.attr[vq.count]) + 16, &hi, 8);
		vq.count++;
	}

	__attribute__((always_inline)) inline void vertex_kick_xyz(uint64_t v) { push_vertex(v, uint32_t(v >> 32), float(field(dec.fog, 56, 8))); }
	__attribute__((always_inline)) inline void vertex_kick_xyzf(uint64_t v) { push_vertex(v, field(v, 32, 24), float(field(v, 56, 8))); }

	// ---------------------------------------------------------------
	// draw_is_degenerate (gs/gs_interface.cpp:2036-2115).
	bool draw_is_degenerate()
	{
		if (degenerate_serial == reg_serial)
			return degenerate_cached;
		degenerate_serial = reg_serial;
		degenerate_cached = compute_draw_is_degenerate();
		return degenerate_cached;
	}

	bool compute_draw_is_degenerate()
	{
		PrimReg prim(regs[R_PRIM]);
		uint64_t sc = ctx_reg(R_SCISSOR_1);
		if (field(sc, 0, 11) > field(sc, 16, 11) || field(sc, 32, 11) > field(sc, 48, 11))
			return true;
		TestReg test(ctx_reg(R_TEST_1));
		if (test.zte && test.ztst == 0)
			return true;
		if (test.ate && test.atst == ATST_NEVER && test.afail == AFAIL_KEEP)
			return true;
		FrameReg frame(ctx_reg(R_FRAME_1));
		ZbufReg zbuf(ctx_reg(R_ZBUF_1));
		uint32_t fbmsk = frame.fbmsk, zmsk = zbuf.zmsk;
		if (frame.psm == PSMCT24 || frame.psm == PSMZ24)
			fbmsk |= 0xffu << 24;
		if (test.ate && test.atst == ATST_NEVER)
		{
			switch (test.afail)
			{
			case AFAIL_ZB_ONLY: fbmsk = 0xffffffffu; break;
			case AFAIL_KEEP: fbmsk = 0xffffffffu; zmsk = 1; break;
			case AFAIL_FB_ONLY: zmsk = 1; break;
			case AFAIL_RGB_ONLY: fbmsk |= 0xffu << 24; break;
			default: break;
			}
		}
		AlphaReg alpha(ctx_reg(R_ALPHA_1));
		if (prim.abe && alpha.d == BLEND_RGB_DEST && alpha.a == alpha.b)
			fbmsk |= 0xffffffu;
		bool ro_color = fbmsk == 0xffffffffu;
		bool ro_depth = zmsk || !test.zte;
		return ro_color && ro_depth;
	}

	bool state_is_z_sensitive()
	{
		TestReg test(ctx_reg(R_TEST_1));
		if (test.zte)
		{
			if (test.has_z_test())
				return true;
			bool implied_z_mask = test.ate && test.atst == ATST_NEVER && test.afail != AFAIL_ZB_ONLY;
			if (!implied_z_mask && ZbufReg(ctx_reg(R_ZBUF_1)).zmsk == 0)
				return true;
		}
		return false;
	}

	// check_frame_buffer_state (gs/gs_interface.cpp:935-1023).  A FRAME / ZBUF
	// change with primitives in the pass moves to a matching instance or opens
	// a new one (the texture cache is checked then), unless short-term cached
	// textures or a full instance table force a flush.
	void check_frame_buffer_state()
	{
		if (!(dirty & DIRTY_FB))
			return;
		dirty &= ~DIRTY_FB;
		const uint64_t frame = ctx_reg(R_FRAME_1), zbuf = ctx_reg(R_ZBUF_1);
		Instance *inst = &instances[current_instance];
		bool fb_delta = !frame_compat(inst->frame, frame);
		bool z_delta = !zbuf_compat(inst->zbuf, zbuf);
		if (primitive_count && (fb_delta || (z_delta && inst->z_sensitive)))
		{
			current_instance = num_instances;
			const bool can_fuse = !has_hazardous_short_term;
			if (can_fuse)
				for (uint32_t i = 0; i < num_instances; i++)
				{
					auto &t = instances[i];
					if (frame_compat(t.frame, frame) && (!t.z_sensitive || zbuf_compat(t.zbuf, zbuf)))
					{
						current_instance = i;
						break;
					}
				}
			if (current_instance == num_instances)
			{
				if (num_instances < PGS_MAX_RENDER_PASS_INSTANCES && can_fuse)
				{
					instances[current_instance] = Instance();
					num_instances++;
					tracker.invalidate_texture_cache(clut_instance);
					if (has_optimized_short_term)
						tracker.invalidate_fb_write_short_term_references();
				}
				else
				{
					flush_pending_transfer(true);
					flush_render_pass(FLUSH_FB_POINTER);
				}
			}
			fb_delta = true;
			z_delta = true;
			last_para_candidate = false;
			inst = &instances[current_instance];
		}
		if (fb_delta)
		{
			const Layout L = psm_layout(field(frame, 24, 6));
			inst->fb_pw = L.pw;
			inst->fb_ph = L.ph;
			inst->frame = frame;
			dirty |= DIRTY_POTENTIAL_FEEDBACK_REGION;
		}
		if (z_delta)
		{
			const Layout L = psm_layout(field(zbuf, 24, 4) | 0x30u);
			inst->z_pw = L.pw;
			inst->z_ph = L.ph;
			inst->zbuf = zbuf;
			dirty |= DIRTY_POTENTIAL_FEEDBACK_REGION;
		}
		// Changing buffers counts as a TEXFLUSH.
		if (fb_delta || z_delta)
			texflush_counter++;
	}

	uint32_t find_state_vector(const pgs_state_vector &s)
	{
		for (uint32_t i = 0; i < state_vectors.size(); i++)
		{
			auto &o = state_vectors[i];
			if (o.combiner == s.combiner && o.blend_mode == s.blend_mode && o.dimx_lo == s.dimx_lo && o.dimx_hi == s.dimx_hi)
				return i;
		}
		state_vectors.push_back(s);
		return uint32_t(state_vectors.size() - 1);
	}

	// drawing_kick_update_state_vector (gs/gs_interface.cpp:1065-1128).
	uint32_t update_state_vector()
	{
		PrimReg prim(regs[R_PRIM]);
		TestReg test(ctx_reg(R_TEST_1));
		AlphaReg alpha(ctx_reg(R_ALPHA_1));
		Tex0Reg tex0(ctx_reg(R_TEX0_1));
		pgs_state_vector s = {};
		if (field(regs[R_DTHE], 0, 1))
		{
			s.blend_mode |= BLEND_MODE_DTHE_BIT;
			s.dimx_lo = uint32_t(regs[R_DIMX]);
			s.dimx_hi = uint32_t(regs[R_DIMX] >> 32);
		}
		if (test.ate && test.atst != ATST_ALWAYS)
		{
			bool implied_z_mask = test.atst == ATST_NEVER && test.afail == AFAIL_FB_ONLY;
			if (!implied_z_mask)
			{
				s.blend_mode |= BLEND_MODE_ATE_BIT;
				s.blend_mode |= test.atst << BLEND_MODE_ATE_MODE_OFFSET;
				s.blend_mode |= test.afail << BLEND_MODE_AFAIL_MODE_OFFSET;
			}
		}
		s.blend_mode |= test.date ? BLEND_MODE_DATE_BIT : 0;
		s.blend_mode |= test.datm ? BLEND_MODE_DATM_BIT : 0;
		if (prim.abe || prim.aa1)
		{
			s.blend_mode |= alpha.a << BLEND_MODE_A_MODE_OFFSET;
			s.blend_mode |= alpha.b << BLEND_MODE_B_MODE_OFFSET;
			s.blend_mode |= alpha.c << BLEND_MODE_C_MODE_OFFSET;
			s.blend_mode |= alpha.d << BLEND_MODE_D_MODE_OFFSET;
		}
		if (prim.abe)
		{
			s.blend_mode |= BLEND_MODE_ABE_BIT;
			s.blend_mode |= field(regs[R_PABE], 0, 1) ? BLEND_MODE_PABE_BIT : 0;
		}
		s.blend_mode |= field(regs[R_COLCLAMP], 0, 1) ? BLEND_MODE_COLCLAMP_BIT : 0;
		s.blend_mode |= field(ctx_reg(R_FBA_1), 0, 1) ? BLEND_MODE_FB_ALPHA_BIT : 0;
		if (prim.tme)
		{
			s.combiner |= COMBINER_TME_BIT;
			s.combiner |= tex0.tcc ? COMBINER_TCC_BIT : 0;
			s.combiner |= tex0.tfx;
		}
		s.combiner |= prim.fge ? COMBINER_FOG_BIT : 0;
		return find_state_vector(s);
	}

	static uint64_t texture_hash(const pgs_texture_desc &d)
	{
		const uint32_t *w = reinterpret_cast<const uint32_t *>(&d);
		uint64_t h = 1469598103934665603ull;
		for (size_t i = 0; i < sizeof(d) / 4; i++)
			h = (h ^ w[i]) * 1099511628211ull;
		return h;
	}

	static uint32_t swizzle_compat_key(uint32_t psm)
	{
		// Formats sharing a swizzle (swizzle_compat_key, gs/shaders/swizzle_utils.h:304-328).
		switch (psm)
		{
		case PSMZ32: return 2;
		case PSMCT16: return 3;
		case PSMZ16: return 4;
		case PSMCT16S: return 5;
		case PSMZ16S: return 6;
		case PSMT8: return 7;
		case PSMT4: return 8;
		case PSMZ24: return 9;
		default: return 1;
		}
	}

	// UV bounding box of a primitive in texels (compute_uv_bb,
	// gs/gs_interface.cpp:2308-2384).  uvs: the vertices' UVs in 1/16 texels.
	void compute_uv_bb(const pgs_vertex_attribute *attr, bool quad, bool conservative, int32_t uv_bb[4],
	                   int32_t (*uvs)[2], bool *needs_perspective)
	{
		const Tex0Reg t0(ctx_reg(R_TEX0_1));
		const Tex1Reg t1(ctx_reg(R_TEX1_1));
		const PrimReg prim(regs[R_PRIM]);
		const float fw = float((1 << int(t0.tw)) * 16), fh = float((1 << int(t0.th)) * 16);
		int32_t local[3][2];
		if (!uvs)
			uvs = local;
		if (needs_perspective)
			*needs_perspective = false;
		const uint32_t nv = quad ? 2 : 3;
		if (prim.fst)
		{
			for (uint32_t i = 0; i < nv; i++)
			{
				uvs[i][0] = attr[i].u;
				uvs[i][1] = attr[i].v;
			}
		}
		else
		{
			if (!quad && needs_perspective && (attr[0].q != attr[1].q || attr[1].q != attr[2].q))
				*needs_perspective = true;
			for (uint32_t i = 0; i < nv; i++)
			{
				const float inv = 1.0f / attr[i].q;
				uvs[i][0] = int32_t(fw * (attr[i].s * inv));
				uvs[i][1] = int32_t(fh * (attr[i].t * inv));
			}
		}
		int32_t lo[2] = { std::min(uvs[0][0], uvs[1][0]), std::min(uvs[0][1], uvs[1][1]) };
		int32_t hi[2] = { std::max(uvs[0][0], uvs[1][0]), std::max(uvs[0][1], uvs[1][1]) };
		if (!quad)
			for (int k = 0; k < 2; k++)
			{
				lo[k] = std::min(lo[k], uvs[2][k]);
				hi[k] = std::max(hi[k], uvs[2][k]);
			}
		if (conservative)
		{
			if (t1.mmag)
			{
				// A linear filter reaches half a texel further.
				for (int k = 0; k < 2; k++)
				{
					lo[k] -= 1 << (SUBPIXEL_BITS - 1);
					hi[k] += (1 << (SUBPIXEL_BITS - 1)) - 1;
				}
			}
			else if (!prim.fst)
			{
				for (int k = 0; k < 2; k++)
				{
					lo[k] -= 1;
					hi[k] += 1;
				}
			}
		}
		uv_bb[0] = lo[0] >> SUBPIXEL_BITS;
		uv_bb[1] = lo[1] >> SUBPIXEL_BITS;
		uv_bb[2] = hi[0] >> SUBPIXEL_BITS;
		uv_bb[3] = hi[1] >> SUBPIXEL_BITS;
		if (!conservative)
		{
			// The last row and column are rarely drawn (raster rules).
			uv_bb[2] = std::max(uv_bb[2] - 1, 0);
			uv_bb[3] = std::max(uv_bb[3] - 1, 0);
		}
	}

	// compute_has_potential_feedback (gs/gs_util.cpp:81-139): can the
	// texture's page range reach the frame or depth buffer's base page.
	void has_potential_feedback(bool &color, bool &depth) const
	{
		const Tex0Reg t0(ctx_reg(R_TEX0_1));
		const ClampReg cl(ctx_reg(R_CLAMP_1));
		const FrameReg fr(ctx_reg(R_FRAME_1));
		const ZbufReg zb(ctx_reg(R_ZBUF_1));
		const Layout L = psm_layout(t0.psm);
		const uint32_t stride = (t0.psm == PSMT4 || t0.psm == PSMT8) ? (t0.tbw >> 1) : t0.tbw;
		uint32_t w = 1u << t0.tw, h = 1u << t0.th;
		const Extent ue = effective_extent(w, cl.wms, cl.minu, cl.maxu, 1);
		const Extent ve = effective_extent(h, cl.wmt, cl.minv, cl.maxv, 1);
		w = ue.base + ue.extent;
		h = ve.base + ve.extent;
		if (w >= 1024 && t0.tbw)
			w = std::min<uint32_t>(w, t0.tbw * BUFFER_WIDTH_SCALE);
		const uint32_t base_block = t0.tbp0, base_page = base_block / BLOCKS_PER_PAGE;
		uint32_t fb_page = fr.fbp, z_page = zb.zbp;
		if (fb_page * BLOCKS_PER_PAGE < base_block)
			fb_page += NUM_PAGES;
		if (z_page * BLOCKS_PER_PAGE < base_block)
			z_page += NUM_PAGES;
		uint32_t last = base_page + ((w - 1) >> L.pw) + ((h - 1) >> L.ph) * stride;
		if (base_block % BLOCKS_PER_PAGE)
			last++;
		last -= base_page;
		fb_page -= base_page;
		z_page -= base_page;
		color = last >= fb_page;
		depth = last >= z_page;
	}

	struct Extent
	{
		uint32_t base, extent;
	};

	// compute_effective_texture_extent (gs/gs_util.cpp:31-79).
	static Extent effective_extent(uint32_t extent, uint32_t wrap, uint32_t lo, uint32_t hi, uint32_t levels)
	{
		uint32_t base = 0;
		if (wrap == WRAP_REGION_CLAMP)
		{
			lo = std::min(lo, hi);
			extent = std::max(hi, lo) - lo + 1;
			if (levels > 1)
			{
				const uint32_t mask = (1u << (levels - 1)) - 1u;
				extent += lo & mask;
				lo &= ~mask;
				extent = (extent + mask) & ~mask;
			}
			base = lo;
		}
		else if (wrap == WRAP_REGION_REPEAT)
		{
			const uint32_t msk = lo, fix = hi;
			if (msk == 0)
			{
				extent = 1;
				base = fix;
			}
			else
			{
				const uint32_t msb = 31u - uint32_t(__builtin_clz(msk));
				const uint32_t lsb = fix ? uint32_t(__builtin_ctz(fix)) : 32u;
				if (lsb > msb)
				{
					extent = std::min(1u << (msb + 1), extent);
					base = fix;
				}
			}
		}
		return { base, extent };
	}

	// update_color_feedback_state (gs/gs_interface.cpp:2141-2306).
	void update_color_feedback_state()
	{
		if (!(dirty & DIRTY_FEEDBACK))
		{
			// In feedback every draw re-evaluates its texture state.
			if (is_color_feedback || is_depth_feedback)
				dirty |= DIRTY_PRIM_TEMPLATE | DIRTY_TEX;
			return;
		}
		dirty &= ~DIRTY_FEEDBACK;
		is_color_feedback = is_depth_feedback = is_awkward_color_feedback = false;
		is_potential_feedback = is_potential_channel_shuffle = false;
		const PrimReg prim(regs[R_PRIM]);
		if (!prim.tme)
			return;
		const Tex0Reg t0(ctx_reg(R_TEX0_1));
		const Tex1Reg t1(ctx_reg(R_TEX1_1));
		const ClampReg cl(ctx_reg(R_CLAMP_1));
		const FrameReg fr(ctx_reg(R_FRAME_1));
		const ZbufReg zb(ctx_reg(R_ZBUF_1));
		const Instance &inst = instances[current_instance];
		// Mipmapping is left alone.
		if (t1.mmin_has_mipmap() && t1.mxl != 0 && !hack_disable_mipmaps)
			return;
		uint32_t tbp0 = t0.tbp0;
		const uint32_t tex_psm = t0.psm;
		if (fr.psm == tex_psm && (tex_psm == PSMCT16 || tex_psm == PSMCT16S || tex_psm == PSMZ16 || tex_psm == PSMZ16S))
			is_potential_channel_shuffle = true;
		// A region clamp can move the effective base onto the framebuffer.
		if (!psm_is_palette(tex_psm))
		{
			const Layout L = psm_layout(tex_psm);
			if (cl.wms == WRAP_REGION_CLAMP && cl.minu != 0)
				tbp0 += BLOCKS_PER_PAGE * (cl.minu >> L.pw);
			if (cl.wmt == WRAP_REGION_CLAMP && cl.minv != 0)
				tbp0 += BLOCKS_PER_PAGE * t0.tbw * (cl.minv >> L.ph);
		}
		const bool eq_color = tbp0 == fr.fbp * BLOCKS_PER_PAGE;
		const bool eq_depth = tbp0 == zb.zbp * BLOCKS_PER_PAGE && (inst.z_sensitive || state_is_z_sensitive());
		if (eq_color && (swizzle_compat_key(tex_psm) != swizzle_compat_key(fr.psm) || t0.tbw != fr.fbw))
		{
			// Same address, different swizzle: no caching makes sense.
			is_color_feedback = true;
			is_awkward_color_feedback = true;
			return;
		}
		if (eq_depth && (swizzle_compat_key(tex_psm) != swizzle_compat_key(zb.psm | 0x30u) || t0.tbw != fr.fbw))
			return;
		if (cl.wms == WRAP_REGION_REPEAT || cl.wmt == WRAP_REGION_REPEAT)
			return;
		if (!eq_color && !eq_depth)
		{
			bool pc = false, pd = false;
			has_potential_feedback(pc, pd);
			bool existing_z_write = inst.z_write && frame_compat(inst.frame, ctx_reg(R_FRAME_1)) &&
			                        zbuf_compat(inst.zbuf, ctx_reg(R_ZBUF_1));
			const bool has_z_write = existing_z_write || (state_is_z_sensitive() && zb.zmsk == 0);
			const uint32_t tex_wm = psm_word_write_mask(tex_psm);
			const uint32_t fb_wm = psm_word_write_mask(FrameReg(inst.frame).psm);
			const uint32_t z_wm = psm_word_write_mask(ZbufReg(inst.zbuf).psm);
			if ((tex_wm & fb_wm) == 0)
				pc = false;
			if ((tex_wm & z_wm) == 0 || !has_z_write)
				pd = false;
			is_potential_feedback = pc || pd;
			if (is_potential_feedback)
			{
				const Layout L = psm_layout(t0.psm);
				potential.base_page = t0.tbp0 / BLOCKS_PER_PAGE;
				potential.pw = L.pw;
				potential.ph = L.ph;
				potential.page_stride = (t0.psm == PSMT4 || t0.psm == PSMT8) ? (t0.tbw >> 1) : t0.tbw;
				potential.width_bias = (t0.tbp0 & (BLOCKS_PER_PAGE - 1)) ? 1 : 0;
				uint32_t safe = UINT32_MAX;
				if (pc)
					safe = std::min<uint32_t>(safe, (fr.fbp - potential.base_page) & (NUM_PAGES - 1));
				if (pd)
					safe = std::min<uint32_t>(safe, (zb.zbp - potential.base_page) & (NUM_PAGES - 1));
				if (potential.width_bias >= safe)
					is_potential_feedback = false;
				else
					potential.max_safe_page = safe - 1 - potential.width_bias;
			}
		}
		else
		{
			is_color_feedback = eq_color && (psm_word_write_mask(tex_psm) & psm_word_write_mask(fr.psm)) != 0;
			is_depth_feedback = eq_depth && (psm_word_write_mask(tex_psm) & psm_word_write_mask(zb.psm)) != 0;
			dirty |= DIRTY_PRIM_TEMPLATE | DIRTY_TEX;
		}
	}

	// deduce_color_feedback_mode (gs/gs_interface.cpp:2388-2471).
	uint32_t deduce_feedback_mode(const pgs_vertex_position *pos, const pgs_vertex_attribute *attr, uint32_t nv,
	                              bool quad, int32_t uv_bb[4], const int32_t *bb)
	{
		if (!(nv == 3 || (quad && nv == 2)))
			return FEEDBACK_NONE;
		if (is_awkward_color_feedback)
			return FEEDBACK_BYPASS_HAZARDS;
		const Tex0Reg t0(ctx_reg(R_TEX0_1));
		const Tex1Reg t1(ctx_reg(R_TEX1_1));
		const ClampReg cl(ctx_reg(R_CLAMP_1));
		const int width = 1 << int(t0.tw), height = 1 << int(t0.th);
		bool needs_perspective = false;
		int32_t uvs[3][2] = {};
		compute_uv_bb(attr, quad, true, uv_bb, uvs, &needs_perspective);
		if (needs_perspective)
			return FEEDBACK_SLICED;
		if (cl.wms == WRAP_REGION_CLAMP)
		{
			if (bb[0] < int(cl.minu) || bb[2] > int(cl.maxu))
				return FEEDBACK_SLICED;
		}
		else if (bb[2] >= width)
			return FEEDBACK_SLICED;
		if (cl.wmt == WRAP_REGION_CLAMP)
		{
			if (bb[1] < int(cl.minv) || bb[3] > int(cl.maxv))
				return FEEDBACK_SLICED;
		}
		else if (bb[3] >= height)
			return FEEDBACK_SLICED;
		int32_t dmin[2], dmax[2];
		for (int k = 0; k < 2; k++)
		{
			const int32_t p0 = k ? pos[0].y : pos[0].x, p1 = k ? pos[1].y : pos[1].x;
			dmin[k] = std::min(uvs[0][k] - p0, uvs[1][k] - p1);
			dmax[k] = std::max(uvs[0][k] - p0, uvs[1][k] - p1);
			if (!quad)
			{
				const int32_t p2 = k ? pos[2].y : pos[2].x;
				dmin[k] = std::min(dmin[k], uvs[2][k] - p2);
				dmax[k] = std::max(dmax[k], uvs[2][k] - p2);
			}
		}
		const int32_t min2 = std::min(dmin[0], dmin[1]), max2 = std::max(dmax[0], dmax[1]);
		if (t1.mmag)
		{
			if (min2 != (1 << (SUBPIXEL_BITS - 1)) || max2 != (1 << (SUBPIXEL_BITS - 1)))
				return FEEDBACK_SLICED;
		}
		else if (min2 < 0 || max2 >= (1 << SUBPIXEL_BITS))
			return FEEDBACK_SLICED;
		return FEEDBACK_PIXEL;
	}

	// Texture page reads (texture_page_rects_read_full / _region /
	// _safe_region, gs/gs_interface.cpp:1151-1206).
	void texture_read_full()
	{
		for (uint32_t l = 0; l < tex_num_rects; l++)
			tracker.mark_texture_read(tex_rects[l]);
	}

	void texture_read_safe_region()
	{
		PageRect r;
		r.base_page = potential.base_page;
		r.page_width = potential.max_safe_page + 1;
		r.page_height = 1;
		r.page_stride = 0;
		r.block_mask = 0xffffffffu;
		r.write_mask = 0xffffffffu;
		tracker.mark_texture_read(r);
	}

	void texture_read_region(const int32_t *uv_bb)
	{
		const Tex0Reg t0(ctx_reg(R_TEX0_1));
		const uint32_t max_px = uint32_t(uv_bb[2]) >> potential.pw, max_py = uint32_t(uv_bb[3]) >> potential.ph;
		if (!(dirty & DIRTY_POTENTIAL_FEEDBACK_REGION))
		{
			// Known to stay below the framebuffer pages.
			if (max_px + max_py * potential.page_stride <= potential.max_safe_page)
				return;
		}
		dirty &= ~DIRTY_POTENTIAL_FEEDBACK_REGION;
		PageRect r;
		r.base_page = t0.tbp0 / BLOCKS_PER_PAGE;
		r.page_width = max_px + 1 + potential.width_bias;
		r.page_height = max_py + 1;
		r.page_stride = potential.page_stride;
		r.block_mask = 0xffffffffu;
		r.write_mask = 0xffffffffu;
		tracker.mark_texture_read(r);
	}

	// mark_render_pass_has_texture_feedback (gs/gs_interface.cpp:909-933).
	void mark_pass_texture_feedback(const Tex0Reg &t0, uint32_t mode)
	{
		if (pass_feedback != PASS_FEEDBACK_NONE && mode != pass_feedback)
			flush_render_pass(FLUSH_TEXTURE_HAZARD);
		if (pass_feedback != PASS_FEEDBACK_NONE &&
		    (t0.psm != pass_feedback_psm || (psm_is_palette(pass_feedback_psm) && pass_feedback_cpsm != t0.cpsm)))
			flush_render_pass(FLUSH_TEXTURE_HAZARD);
		if (pass_feedback == PASS_FEEDBACK_NONE)
		{
			pass_feedback = mode;
			pass_feedback_psm = t0.psm;
			pass_feedback_cpsm = psm_is_palette(t0.psm) ? t0.cpsm : 0;
		}
		if (pass_feedback == PASS_FEEDBACK_DEPTH)
			instances[current_instance].z_feedback = true;
	}

	// Texture of the current context (drawing_kick_update_texture,
	// gs/gs_interface.cpp:1254-1800).  The descriptor keeps what the decode
	// depends on; hazard reads follow the reference's caching of the texture
	// (long-term, short-term for feedback and very large images).  A draw the
	// reference would sample from the framebuffer tile itself (pixel
	// feedback) is drawn here as an ordinary texture read, checked like one.
	uint32_t update_texture(uint32_t feedback_mode, const int32_t *uv_bb, const int32_t *bb)
	{
		if (!(dirty & DIRTY_TEX) && last_texture_index != UINT32_MAX)
			return last_texture_index;
		dirty &= ~DIRTY_TEX;
		const PrimReg prim(regs[R_PRIM]);
		const Tex0Reg t(ctx_reg(R_TEX0_1));
		const ClampReg c(ctx_reg(R_CLAMP_1));
		const Tex1Reg tex1(ctx_reg(R_TEX1_1));
		const FrameReg fr(ctx_reg(R_FRAME_1));
		const uint64_t texa = regs[R_TEXA];
		const bool pixel_feedback = feedback_mode == FEEDBACK_PIXEL;
		if (pixel_feedback)
		{
			mark_pass_texture_feedback(t, is_color_feedback ? PASS_FEEDBACK_COLOR : PASS_FEEDBACK_DEPTH);
			feedback_mode = FEEDBACK_BYPASS_HAZARDS;
		}

		pgs_texture_desc d = {};
		d.tbp0 = t.tbp0;
		d.tbw = t.tbw;
		d.psm = t.psm;
		d.tw_log2 = std::min<uint32_t>(t.tw, 10);
		d.th_log2 = std::min<uint32_t>(t.th, 10);
		const uint32_t cpsm = t.cpsm == PSMCT24 ? PSMCT32 : t.cpsm;
		uint32_t csa_mask = 0;
		if (psm_is_palette(t.psm))
		{
			d.cpsm = cpsm;
			d.csa = cpsm == PSMCT32 ? (t.csa & 15) : t.csa;
			d.clut_instance = clut_instance;
			if (cpsm != PSMCT32)
			{
				d.aem = field(texa, 15, 1);
				d.ta0 = field(texa, 0, 8);
				d.ta1 = field(texa, 32, 8);
			}
			// The newest CLUT load is now in use (mark_clut_read).
			if (clut_instance == ring_next)
				ring_last_read = true;
			csa_mask = (t.psm == PSMT8 || t.psm == PSMT8H) ? 0xffffu : 1u;
			csa_mask <<= d.csa;
			if (cpsm == PSMCT32)
			{
				csa_mask &= 0xffffu;
				csa_mask |= csa_mask << 16;
			}
		}
		else if (t.psm != PSMCT32 && t.psm != PSMZ32)
		{
			d.aem = field(texa, 15, 1);
			d.ta0 = field(texa, 0, 8);
			d.ta1 = field(texa, 32, 8);
		}

		uint32_t wms = c.wms, wmt = c.wmt, minu = c.minu, maxu = c.maxu, minv = c.minv, maxv = c.maxv;
		bool long_term = true;
		if (feedback_mode == FEEDBACK_SLICED)
		{
			auto overlap_empty = [](int32_t x0, int32_t y0, int32_t x1, int32_t y1) { return x0 > x1 || y0 > y1; };
			if (prim.prim == PRIM_SPRITE)
			{
				long_term = !current_is_channel_shuffle;
				if (long_term && fr.fbw >= 4 && uv_bb[2] - uv_bb[0] < 16 && uv_bb[3] - uv_bb[1] < 16 &&
				    bb[2] - bb[0] < 16 && bb[3] - bb[1] < 16)
				{
					const int32_t hx0 = std::max(uv_bb[0], bb[0]), hy0 = std::max(uv_bb[1], bb[1]);
					const int32_t hx1 = std::min(uv_bb[2], bb[2]), hy1 = std::min(uv_bb[3], bb[3]);
					long_term = (hx1 + 64 < hx0) || (hy1 + 64 < hy0);
				}
				if (long_term && tex1.mmag)
				{
					// In-place blur at a tiny bias.
					const int u_off = std::abs(uv_bb[0] - bb[0]), v_off = std::abs(uv_bb[1] - bb[1]);
					const int u_size = uv_bb[2] - uv_bb[0] - 2, v_size = uv_bb[3] - uv_bb[1] - 2;
					if (u_off <= 1 && v_off <= 1 && u_size == bb[2] - bb[0] && v_size == bb[3] - bb[1])
						long_term = false;
				}
			}
			else if (wms == WRAP_REGION_CLAMP && wmt == WRAP_REGION_CLAMP)
			{
				long_term = overlap_empty(std::max(int32_t(minu), bb[0]), std::max(int32_t(minv), bb[1]),
				                          std::min(int32_t(maxu), bb[2]), std::min(int32_t(maxv), bb[3]));
			}
			else if (last_para_candidate)
			{
				long_term = overlap_empty(std::max(uv_bb[0], bb[0]), std::max(uv_bb[1], bb[1]),
				                          std::min(uv_bb[2], bb[2]), std::min(uv_bb[3], bb[3]));
			}
			else
				long_term = false;
		}
		else if (feedback_mode == FEEDBACK_BYPASS_HAZARDS)
			long_term = false;

		const uint32_t width = 1u << t.tw, height = 1u << t.th;
		if (is_potential_feedback && width > t.tbw * BUFFER_WIDTH_SCALE && t.tbw != 0 && height > (1u << psm_layout(t.psm).ph))
		{
			// A texture wider than its stride: clamp to the stride.
			if (wms == WRAP_CLAMP || wms == WRAP_REPEAT)
			{
				wms = WRAP_REGION_CLAMP;
				minu = 0;
				maxu = t.tbw * BUFFER_WIDTH_SCALE - 1;
			}
			else if (wms == WRAP_REGION_CLAMP)
			{
				minu = std::min<uint32_t>(minu, t.tbw * BUFFER_WIDTH_SCALE - 1);
				maxu = std::min<uint32_t>(maxu, t.tbw * BUFFER_WIDTH_SCALE - 1);
			}
		}
		if (feedback_mode == FEEDBACK_SLICED && long_term && wms != WRAP_REGION_REPEAT && wmt != WRAP_REGION_REPEAT)
		{
			// Narrow to the sampled box.
			if (wms == WRAP_REGION_CLAMP)
			{
				minu = uint32_t(std::max<int>(int(minu), std::min<int>(uv_bb[0], int(maxu))));
				maxu = uint32_t(std::min<int>(int(maxu), std::max<int>(uv_bb[2], int(minu))));
			}
			else if (wms == WRAP_CLAMP || (uv_bb[2] < int(width) && uv_bb[0] >= 0))
			{
				wms = WRAP_REGION_CLAMP;
				minu = uint32_t(std::max<int>(0, uv_bb[0]));
				maxu = uint32_t(std::min<int>(int(width) - 1, uv_bb[2]));
			}
			if (wmt == WRAP_REGION_CLAMP)
			{
				minv = uint32_t(std::max<int>(int(minv), std::min<int>(uv_bb[1], int(maxv))));
				maxv = uint32_t(std::min<int>(int(maxv), std::max<int>(uv_bb[3], int(minv))));
			}
			else if (wmt == WRAP_CLAMP || (uv_bb[3] < int(height) && uv_bb[1] >= 0))
			{
				wmt = WRAP_REGION_CLAMP;
				minv = uint32_t(std::max<int>(0, uv_bb[1]));
				maxv = uint32_t(std::min<int>(int(height) - 1, uv_bb[3]));
			}
		}
		// Only the region modes stay in the descriptor; plain REPEAT and CLAMP
		// read as CLAMP with zero bounds and the primitive's sampler bits pick
		// between them (gs/gs_interface.cpp:1514-1528), so both share a decode.
		if (wms < WRAP_REGION_CLAMP)
		{
			wms = WRAP_CLAMP;
			minu = maxu = 0;
		}
		if (wmt < WRAP_REGION_CLAMP)
		{
			wmt = WRAP_CLAMP;
			minv = maxv = 0;
		}
		d.wms = wms;
		d.wmt = wmt;
		d.minu = minu & 0x3ff;
		d.maxu = maxu & 0x3ff;
		d.minv = minv & 0x3ff;
		d.maxv = maxv & 0x3ff;

		// Mip levels sampled (compute_effective_texture_rect,
		// gs/gs_renderer.cpp:1235-1265); MXL only counts with a mipmapping MMIN.
		const uint32_t mxl = (tex1.mmin_has_mipmap() && !hack_disable_mipmaps) ? tex1.mxl : 0;
		d.mxl = mxl;
		const uint32_t max_levels = std::min<uint32_t>(7, std::min(d.tw_log2, d.th_log2) + 1);
		d.levels = std::min<uint32_t>(mxl + 1, max_levels);
		const Extent ue = effective_extent(1u << d.tw_log2, d.wms, d.minu, d.maxu, d.levels);
		const Extent ve = effective_extent(1u << d.th_log2, d.wmt, d.minv, d.maxv, d.levels);
		uint32_t level_base[7] = { t.tbp0 }, level_stride[7] = { t.tbw };
		for (uint32_t l = 1; l < d.levels; l++)
		{
			uint64_t m = ctx_reg(l <= 3 ? R_MIPTBP1_1 : R_MIPTBP2_1);
			uint32_t slot = (l - 1) % 3;
			level_base[l] = field(m, 20 * slot, 14);
			level_stride[l] = field(m, 20 * slot + 14, 6);
			d.mip[l - 1] = level_base[l] | (level_stride[l] << 16);
		}
		tex_num_rects = d.levels;
		for (uint32_t l = 0; l < d.levels; l++)
			tex_rects[l] = compute_page_rect(level_base[l], ue.base >> l, ve.base >> l, ue.extent >> l, ve.extent >> l,
			                                 level_stride[l], t.psm);

		// The reference reads a pixel-feedback texel from the tile it shades;
		// read through a texture, it must not miss framebuffer writes of the
		// pass.
		if (pixel_feedback)
			texture_read_full();

		// Super-sampled texture: a sprite reading, at 8+ bits per texel, pages
		// that a pass wrote (gs/gs_interface.cpp:1593-1601).
		if (d.levels == 1 && ssaa_textures && psm_bits_per_pixel(t.psm) >= 8 && prim.prim == PRIM_SPRITE &&
		    tracker.texture_may_super_sample(tex_rects[0]))
			d.samples = 1u << (sampling_rate_x_log2 + sampling_rate_y_log2);

		const uint64_t hash = texture_hash(d);
		auto find = [&]() -> TexEntry * {
			auto it = tex_entries.find(hash);
			return it == tex_entries.end() ? nullptr : &it->second;
		};
		TexEntry *cached = find();
		const bool skip_hazards = cached && cached->valid && cached->valid_at == texflush_counter &&
		                          feedback_mode == FEEDBACK_NONE;
		if (!skip_hazards)
		{
			if (is_potential_feedback)
			{
				long_term = false;
				texture_read_region(uv_bb);
			}
			else if (long_term)
				texture_read_full();
			// The pass may have ended: look again.
			cached = find();
			if (cached && cached->valid && cached->long_term && !long_term)
			{
				texture_read_full();
				cached = find();
			}
		}
		if (!long_term)
			has_hazardous_short_term = true;

		if (last_texture_index != UINT32_MAX && !textures.empty() &&
		    memcmp(&last_texture_desc, &d, sizeof(d)) == 0)
		{
			last_texture_valid_at = texflush_counter;
			if (cached && cached->valid)
				cached->valid_at = texflush_counter;
			return last_texture_index;
		}

		uint32_t index;
		if (cached && cached->valid)
			index = cached->index;
		else
		{
			if (is_potential_feedback)
				texture_read_safe_region();
			else if (!long_term || skip_hazards)
				texture_read_full();
			if (long_term)
			{
				// Very large images are held for this pass only.
				const uint32_t pixels = ue.extent * ve.extent;
				const uint32_t threshold = tracker.texture_may_super_sample(tex_rects[0]) ? 128 * 128 : 512 * 512;
				if (d.levels == 1 && (pixels > threshold || ue.extent >= 1024 || ve.extent >= 1024))
				{
					long_term = false;
					has_optimized_short_term = true;
				}
			}
			if (!tracker.find_texture(hash))
			{
				if (long_term)
					tracker.register_texture(tex_rects, d.levels, csa_mask, clut_instance, hash);
				else
					tracker.register_short_term_texture(tex_rects, d.levels, hash);
			}
			index = uint32_t(textures.size());
			if (cached)
			{
				cached->valid_at = texflush_counter;
				cached->index = index;
				cached->valid = true;
			}
			else
				tex_entries[hash] = { index, texflush_counter, long_term, true };
			textures.push_back(d);
			for (uint32_t l = 0; l < d.levels; l++)
				mark_pass_texture(tex_rects[l]);
		}
		last_texture_desc = d;
		last_texture_index = index;
		last_texture_valid_at = texflush_counter;
		texflush_pending = false;
		return index;
	}

	// drawing_kick_update_state (gs/gs_interface.cpp:1804-1968): the
	// primitive template, rebuilt when state it depends on changed.
	// bb: the scissored box of the primitive being drawn.
	void update_state(uint32_t feedback_mode, const int32_t *uv_bb, const int32_t *bb)
	{
		if (!(dirty & DIRTY_PRIM_TEMPLATE))
			return;
		dirty &= ~DIRTY_PRIM_TEMPLATE;
		tpl_serial++;
		PrimReg prim(regs[R_PRIM]);
		TestReg test(ctx_reg(R_TEST_1));
		AlphaReg alpha(ctx_reg(R_ALPHA_1));
		ZbufReg zbuf(ctx_reg(R_ZBUF_1));
		uint32_t state = 0, tex = 0, tex2 = 0;

		if (prim.tme)
		{
			Tex1Reg tex1(ctx_reg(R_TEX1_1));
			ClampReg clamp(ctx_reg(R_CLAMP_1));
			uint32_t index = update_texture(feedback_mode, uv_bb, bb);
			tex = index;
			if (textures[index].samples > 1)
			{
				// Per-sample layers; palette textures under region repeat map
				// sample to sample (gs/gs_interface.cpp:1786-1791,1822-1831).
				tex |= TEX_PER_SAMPLE_BIT;
				if (psm_is_palette(textures[index].psm) && (clamp.wms == WRAP_REGION_REPEAT || clamp.wmt == WRAP_REGION_REPEAT))
					tex |= TEX_SAMPLE_MAPPING_BIT;
				has_ss_textures = true;
			}
			tex |= tex1.mmag ? TEX_SAMPLER_MAG_LINEAR_BIT : 0;
			tex |= (clamp.wms == WRAP_CLAMP || clamp.wms == WRAP_REGION_CLAMP) ? TEX_SAMPLER_CLAMP_S_BIT : 0;
			tex |= (clamp.wmt == WRAP_CLAMP || clamp.wmt == WRAP_REGION_CLAMP) ? TEX_SAMPLER_CLAMP_T_BIT : 0;
			if (tex1.mmin_has_mipmap() && !hack_disable_mipmaps)
			{
				tex2 = tex1.lcm;
				tex2 |= tex1.l << 1;
				tex2 |= tex1.k << 3;
				tex |= tex1.mxl << TEX_MAX_MIP_LEVEL_OFFSET;
				has_mipmap = has_mipmap || tex1.mxl != 0;
				switch (tex1.mmin)
				{
				case 1: tex |= TEX_SAMPLER_MIN_LINEAR_BIT; break;
				case 3: tex |= TEX_SAMPLER_MIPMAP_LINEAR_BIT; break;
				case 4: tex |= TEX_SAMPLER_MIN_LINEAR_BIT; break;
				case 5: tex |= TEX_SAMPLER_MIN_LINEAR_BIT | TEX_SAMPLER_MIPMAP_LINEAR_BIT; break;
				default: break;
				}
			}
			else
			{
				tex2 = TEX2_FIXED_LOD_BIT;
			}
		}

		state = update_state_vector();

		if (test.zte)
		{
			if (test.has_z_test())
			{
				state |= 1u << STATE_BIT_Z_TEST;
				state |= test.ztst == 3 ? (1u << STATE_BIT_Z_TEST_GREATER) : 0;
			}
			bool implied_z_mask = test.ate && test.atst == ATST_NEVER && test.afail != AFAIL_ZB_ONLY;
			if (!implied_z_mask && zbuf.zmsk == 0)
				state |= 1u << STATE_BIT_Z_WRITE;
		}

		bool needs_previous = false;
		if (prim.abe || prim.aa1)
		{
			if (alpha.a == BLEND_RGB_DEST || alpha.b == BLEND_RGB_DEST || alpha.c == BLEND_ALPHA_DEST ||
			    alpha.d == BLEND_RGB_DEST)
				needs_previous = true;
		}
		if (test.date)
			needs_previous = true;
		else if (test.ate && test.atst != ATST_ALWAYS)
		{
			bool can_write_z = (state & (1u << STATE_BIT_Z_WRITE)) != 0;
			bool can_mask_color = test.afail != AFAIL_FB_ONLY;
			bool can_mask_z = can_write_z && test.afail != AFAIL_ZB_ONLY;
			if (can_mask_color || can_mask_z)
				needs_previous = true;
		}
		if (!needs_previous)
			state |= 1u << STATE_BIT_OPAQUE;

		if (prim.enables_aa1())
		{
			state |= 1u << STATE_BIT_MULTISAMPLE;
			has_aa1 = true;
		}

		uint32_t msk = field(regs[R_SCANMSK], 0, 2);
		if (msk >= 2)
		{
			state |= 1u << (STATE_BIT_SCANMSK_EVEN + msk - 2);
			has_scanmsk = true;
			// A SCANMSK primitive taller than 400 rows interleaves fields
			// itself: progressive read-out is off for the next 4 vsyncs.
			if (bb[1] + 400 < bb[3])
				complex_scanmsk_timeout = 4;
		}

		if (!prim.fst)
			state |= 1u << STATE_BIT_PERSPECTIVE;
		if (prim.iip)
			state |= 1u << STATE_BIT_IIP;
		if (prim.fix)
			state |= 1u << STATE_BIT_FIX;

		tpl_state = state;
		tpl_tex = tex;
		tpl_tex2 = tex2;
	}

	// ---------------------------------------------------------------
	// Drawing kick (gs/gs_interface.cpp:2473-2943).
	// Vertex side of the drawing kick: a kick that completes a primitive
	// hands its vertices, newest first, to the state side (draw), which
	// checks for degenerate state and appends; every kick ends in post_kick
	// on the state side.
	template <class Sink>
	__attribute__((always_inline)) inline void drawing_kick(Sink &s, bool adc)
	{
		auto &vq = dec.vq;
		uint32_t type = field(dec.prim, 0, 3);
		uint32_t nv;
		bool list = false, fan = false, quad = false;
		switch (type)
		{
		case PRIM_POINT: nv = 1; list = true; quad = true; break;
		case PRIM_LINE_LIST: nv = 2; list = true; break;
		case PRIM_LINE_STRIP: nv = 2; break;
		case PRIM_TRI_LIST: nv = 3; list = true; break;
		case PRIM_TRI_STRIP: nv = 3; break;
		case PRIM_TRI_FAN: nv = 3; fan = true; break;
		case PRIM_SPRITE: nv = 2; list = true; quad = true; break;
		default:
			vq.count = 0;
			s.kick();
			return;
		}

		if (vq.count < nv)
		{
			s.kick();
			return;
		}
		if (!adc)
		{
			const DrawSlot d = s.begin_draw(nv, quad);
			for (uint32_t i = 0; i < nv && i < 3; i++)
				copy_vertex(d.pos[i], d.attr[i], vq.pos[vq.count - 1 - i], vq.attr[vq.count - 1 - i]);
			s.end_draw();
		}
		else
			s.kick();
		if (fan)
		{
			copy_vertex(vq.pos[1], vq.attr[1], vq.pos[2], vq.attr[2]);
			vq.count = 2;
		}
		else if (list)
			vq.count = 0;
	}

	// State side of a drawing kick that completes a primitive.
	void draw(uint32_t nv, bool quad, const pgs_vertex_position *vp, const pgs_vertex_attribute *va)
	{
		if (!draw_is_degenerate())
			append(nv, quad, vp, va);
		post_kick();
	}

	// post_draw_kick_handler (gs/gs_interface.cpp:2930-2943).  Runs after
	// every kick: the checks are inline, the flushes out of line.
	__attribute__((always_inline)) inline void post_kick()
	{
		if (__builtin_expect(pending_palette_updates >= PGS_CLUT_INSTANCES - 1 ||
		                     primitive_count >= PGS_MAX_PRIMITIVES_PER_FLUSH || textures.size() >= PGS_MAX_TEXTURES ||
		                     state_vectors.size() >= PGS_MAX_STATE_VECTORS || tracker.memory_pressure(), 0))
			post_kick_flush();
	}

	__attribute__((noinline)) void post_kick_flush()
	{
		if (pending_palette_updates >= PGS_CLUT_INSTANCES - 1 || primitive_count >= PGS_MAX_PRIMITIVES_PER_FLUSH ||
		    textures.size() >= PGS_MAX_TEXTURES || state_vectors.size() >= PGS_MAX_STATE_VECTORS)
		{
			flush_pending_transfer(true);
			flush_render_pass(FLUSH_OVERFLOW);
		}
		tracker.flush_if_memory_pressure();
	}

	// Pages of the instance's box in its frame or depth buffer (compute_fb_rect /
	// compute_z_rect, gs/gs_interface.cpp:1970-2034): block-exact inside one
	// page, whole pages otherwise.
	PageRect instance_rect(const Instance &inst, bool depth) const
	{
		const FrameReg fr(inst.frame);
		const ZbufReg zb(inst.zbuf);
		const uint32_t pw = depth ? inst.z_pw : inst.fb_pw, ph = depth ? inst.z_ph : inst.fb_ph;
		const uint32_t base = depth ? zb.zbp : fr.fbp;
		const uint32_t psm = depth ? (zb.psm | 0x30u) : fr.psm;
		const int32_t px0 = inst.bb[0] >> pw, py0 = inst.bb[1] >> ph, px1 = inst.bb[2] >> pw, py1 = inst.bb[3] >> ph;
		PageRect r;
		r.base_page = base;
		r.page_width = uint32_t(px1 - px0 + 1);
		r.page_height = uint32_t(py1 - py0 + 1);
		if (r.page_width == 1 && r.page_height == 1)
			return compute_page_rect(base * BLOCKS_PER_PAGE, uint32_t(inst.bb[0]), uint32_t(inst.bb[1]),
			                         uint32_t(inst.bb[2] - inst.bb[0] + 1), uint32_t(inst.bb[3] - inst.bb[1] + 1),
			                         fr.fbw, psm);
		r.page_stride = fr.fbw;
		r.base_page += uint32_t(px0) + uint32_t(py0) * r.page_stride;
		r.block_mask = 0xffffffffu;
		r.write_mask = psm_word_write_mask(depth ? zb.psm : fr.psm);
		return r;
	}

	// vp / va: the primitive's vertices, newest first.
	void append(uint32_t nv, bool quad, const pgs_vertex_position *vp, const pgs_vertex_attribute *va)
	{
		const DrawConsts &D = draw_consts();
		// Triangles and sprites are read from the records as handed in and
		// copied once, into the pass (sp / sa point at them).  Points and
		// lines, whose unused vertices read as zero, and primitives that the
		// frame-buffer wrap below moves go through the local copies.
		pgs_vertex_position pos[3];
		pgs_vertex_attribute attr[3];
		const pgs_vertex_position *sp = vp;
		const pgs_vertex_attribute *sa = va;
		if (nv == 1 || (nv == 2 && !quad))
		{
			pos[2] = {};
			attr[1] = {};
			attr[2] = {};
			copy_vertex(pos[0], attr[0], vp[0], va[0]);
			if (nv == 1)
			{
				pos[0].x -= (1 << (SUBPIXEL_BITS - 1)) - 1;
				pos[0].y -= (1 << (SUBPIXEL_BITS - 1)) - 1;
				pos[1] = pos[0];
				pos[1].x += 1 << SUBPIXEL_BITS;
				pos[1].y += 1 << SUBPIXEL_BITS;
			}
			else
				copy_vertex(pos[1], attr[1], vp[1], va[1]);
			sp = pos;
			sa = attr;
		}

		bool is_line = !quad && nv == 2;
		// The box from the records as handed in, not from the copies just
		// stored (reading a field of a 16-byte store right after it can wait
		// for the store to retire).
		int32_t lo[2], hi[2];
		if (nv == 1)
		{
			lo[0] = vp[0].x - ((1 << (SUBPIXEL_BITS - 1)) - 1);
			lo[1] = vp[0].y - ((1 << (SUBPIXEL_BITS - 1)) - 1);
			hi[0] = lo[0] + (1 << SUBPIXEL_BITS);
			hi[1] = lo[1] + (1 << SUBPIXEL_BITS);
		}
		else
		{
			lo[0] = std::min(vp[0].x, vp[1].x);
			lo[1] = std::min(vp[0].y, vp[1].y);
			hi[0] = std::max(vp[0].x, vp[1].x);
			hi[1] = std::max(vp[0].y, vp[1].y);
			if (!quad && !is_line)
			{
				lo[0] = std::min(lo[0], vp[2].x);
				lo[1] = std::min(lo[1], vp[2].y);
				hi[0] = std::max(hi[0], vp[2].x);
				hi[1] = std::max(hi[1], vp[2].y);
			}
		}
		const int32_t pre_lo[2] = { lo[0], lo[1] }, pre_hi[2] = { hi[0], hi[1] };
		hi[0] -= 1;
		hi[1] -= 1;
		lo[0] += D.snap;
		lo[1] += D.snap;
		lo[0] >>= SUBPIXEL_BITS;
		lo[1] >>= SUBPIXEL_BITS;
		hi[0] >>= SUBPIXEL_BITS;
		hi[1] >>= SUBPIXEL_BITS;
		if (is_line || D.line_aa1)
		{
			lo[0] -= 1; lo[1] -= 1;
			hi[0] += 1; hi[1] += 1;
		}

		const FrameReg &frame = D.frame;
		const int32_t sci_hi_x_fb = D.sci_hi_x_fb;
		const bool can_wrap = D.can_wrap;
		int32_t bb[4] = { std::max(lo[0], D.sci_lo[0]), std::max(lo[1], D.sci_lo[1]),
		                  std::min(hi[0], D.sci_hi[0]), std::min(hi[1], D.sci_hi[1]) };
		if (bb[2] < bb[0] || bb[3] < bb[1])
			return;

		// The scissor and degenerate state have been consumed.
		dirty &= ~(DIRTY_SCISSOR | DIRTY_DEGENERATE);

		// A right triangle that completes the rectangle of the previous one,
		// with no state change in between, turns that one into a
		// parallelogram (gs/gs_interface.cpp:2569-2602).
		bool para_candidate = false;
		if (nv == 3 && !quad)
		{
			PrimReg prim(regs[R_PRIM]);
			uint32_t order[3];
			// Triangles: pos / attr are still copies of vp / va; the tests read
			// the records as handed in (see the box above).
			para_candidate = parallelogram_candidate(vp, va, pre_lo, pre_hi, prim, order);
			if (dirty == 0 && para_candidate && last_para_candidate && primitive_count &&
			    forms_parallelogram(vp, va, order, positions + 3 * (primitive_count - 1),
			                        attributes + 3 * (primitive_count - 1), last_para_order, prim))
			{
				prims[primitive_count - 1].state |= (1u << STATE_BIT_PARALLELOGRAM) |
				                                    (last_para_order[0] << STATE_PARALLELOGRAM_PROVOKING_OFFSET);
				last_para_candidate = false;
				return;
			}
			memcpy(last_para_order, order, sizeof(order));
		}

		// Texture feedback against the frame / depth buffer
		// (drawing_kick_append, gs/gs_interface.cpp:2604-2630).
		if ((dirty & DIRTY_FEEDBACK) || is_color_feedback || is_depth_feedback)
			update_color_feedback_state();
		uint32_t feedback_mode = FEEDBACK_NONE;
		int32_t uv_bb[4] = {};
		if (is_color_feedback || is_depth_feedback)
		{
			last_para_candidate = para_candidate;
			feedback_mode = deduce_feedback_mode(sp, sa, nv, quad, uv_bb, bb);
		}
		else if (is_potential_feedback || (is_potential_channel_shuffle && quad))
			compute_uv_bb(sa, quad, false, uv_bb, nullptr, nullptr);
		current_is_channel_shuffle = false;
		if (quad && is_potential_channel_shuffle)
		{
			// A channel shuffle copies within one 8-pixel column at an X offset of 8.
			if ((bb[0] & ~7) == (bb[2] & ~7) && (uv_bb[0] ^ 8) == bb[0] && uv_bb[1] == bb[1])
				current_is_channel_shuffle = true;
		}

		// Flush a pending partial upload before reading textures.
		if (D.tme && xfer.active && xfer.payload.size() > xfer.flushed_qwords)
			flush_pending_transfer(true);

		check_frame_buffer_state();

		// A held texture is checked again after a TEXFLUSH or in feedback
		// (gs/gs_interface.cpp:2646-2670).
		if (D.tme && !(dirty & DIRTY_TEX))
		{
			if (texflush_pending)
			{
				texflush_counter++;
				texflush_pending = false;
			}
			if (texflush_counter != last_texture_valid_at || feedback_mode != FEEDBACK_NONE)
			{
				if (is_potential_feedback)
					texture_read_region(uv_bb);
				else
					texture_read_full();
				if (!(dirty & DIRTY_TEX))
					last_texture_valid_at = texflush_counter;
			}
		}

		if (dirty & DIRTY_PRIM_TEMPLATE)
			update_state(feedback_mode, uv_bb, bb);

		auto &inst = instances[current_instance];
		const uint32_t tex = tpl_tex, tex2 = tpl_tex2, alpha_word = D.alpha_word, fbmsk = frame.fbmsk,
		               fogcol = D.fogcol;
		uint32_t state = tpl_state;
		if (quad)
		{
			state |= (1u << STATE_BIT_PARALLELOGRAM) | (1u << STATE_BIT_SPRITE) |
			         (1u << STATE_BIT_SNAP_RASTER) | (1u << STATE_BIT_SNAP_ATTRIBUTE);
			state &= ~(1u << STATE_BIT_MULTISAMPLE);
		}
		else if (is_line)
		{
			state |= (1u << STATE_BIT_PARALLELOGRAM) | (1u << STATE_BIT_LINE);
			if (state & (1u << STATE_BIT_MULTISAMPLE))
				state &= ~(1u << STATE_BIT_Z_WRITE);
		}
		if (nv == 1)
			state |= (1u << STATE_BIT_FIX) | (1u << STATE_BIT_SNAP_RASTER) | (1u << STATE_BIT_SNAP_ATTRIBUTE);
		state |= current_instance << STATE_VERTEX_RENDER_PASS_INSTANCE_OFFSET;

		// The pages the instance writes are marked when its damage grows
		// (gs/gs_interface.cpp:2712-2816): from no depth to read-only depth, to
		// depth writes, to more colour bits written, or a larger box.
		bool expands = false;
		const bool z_sens = D.z_sens;
		if (!inst.z_sensitive && z_sens)
		{
			inst.z_sensitive = true;
			expands = true;
		}
		if (z_sens && D.zb.zmsk == 0 && !inst.z_write)
		{
			inst.z_write = true;
			// Depth writes may create a feedback that was not there.
			dirty |= DIRTY_FEEDBACK;
			expands = true;
		}
		const uint32_t write_mask = ~frame.fbmsk;
		if ((write_mask & inst.color_write_mask) != write_mask)
		{
			inst.color_write_mask |= write_mask;
			expands = true;
		}

		if (can_wrap && bb[0] > sci_hi_x_fb)
		{
			if (sp != pos)
			{
				for (uint32_t i = 0; i < nv; i++)
					copy_vertex(pos[i], attr[i], sp[i], sa[i]);
				for (uint32_t i = nv; i < 3; i++)
				{
					pos[i] = {};
					attr[i] = {};
				}
				sp = pos;
				sa = attr;
			}
			Layout L = psm_layout(frame.psm);
			int32_t x_off = -int32_t(frame.fbw << L.pw);
			int32_t y_off = int32_t(1u << L.ph);
			while (bb[0] > sci_hi_x_fb)
			{
				bb[0] += x_off; bb[2] += x_off;
				bb[1] += y_off; bb[3] += y_off;
				for (uint32_t i = 0; i < nv; i++)
				{
					pos[i].x += x_off << SUBPIXEL_BITS;
					pos[i].y += y_off << SUBPIXEL_BITS;
				}
			}
			bb[2] = std::min(bb[2], sci_hi_x_fb);
			bb[0] = std::max(bb[0], 0);
			if (bb[2] < bb[0])
				return;
		}
		else if (can_wrap)
		{
			bb[2] = std::min(bb[2], sci_hi_x_fb);
		}

		if (bb[0] < inst.bb[0]) { expands = true; inst.bb[0] = bb[0]; }
		if (bb[1] < inst.bb[1]) { expands = true; inst.bb[1] = bb[1]; }
		if (bb[2] > inst.bb[2]) { expands = true; inst.bb[2] = bb[2]; }
		if (bb[3] > inst.bb[3]) { expands = true; inst.bb[3] = bb[3]; }
		if (expands)
		{
			PageRect fb = instance_rect(inst, false);
			fb.write_mask &= inst.color_write_mask;
			tracker.mark_fb_write(fb);
			if (inst.z_sensitive)
			{
				const PageRect z = instance_rect(inst, true);
				if (inst.z_write)
					tracker.mark_fb_write(z);
				else
					tracker.mark_fb_read(z);
			}
		}

		// The record is assembled in registers and stored as two 16-byte
		// words: bb, state | tex, tex2 | alpha, fbmsk | fogcol.
		const uint32_t n = primitive_count;
		// The pass's buffers are written once, front to back: ask for the
		// lines a few records ahead (a prefetch past the end does not fault).
		prefetch_for_write(prims, (n + ARENA_PREFETCH_RECORDS) * sizeof(pgs_primitive_attribute));
		prefetch_for_write(positions, 3 * (n + ARENA_PREFETCH_RECORDS) * sizeof(pgs_vertex_position));
		prefetch_for_write(attributes, 3 * (n + ARENA_PREFETCH_RECORDS) * sizeof(pgs_vertex_attribute));
		prefetch_for_write(attributes, 3 * (n + ARENA_PREFETCH_RECORDS) * sizeof(pgs_vertex_attribute) + 64);
		{
			static_assert(sizeof(pgs_primitive_attribute) == 32 && offsetof(pgs_primitive_attribute, state) == 8 &&
			              offsetof(pgs_primitive_attribute, fogcol) == 28, "primitive record layout");
			Word2 w0, w1;
			w0[0] = uint64_t(uint16_t(bb[0])) | (uint64_t(uint16_t(bb[1])) << 16) |
			        (uint64_t(uint16_t(bb[2])) << 32) | (uint64_t(uint16_t(bb[3])) << 48);
			w0[1] = uint64_t(state) | (uint64_t(tex) << 32);
			w1[0] = uint64_t(tex2) | (uint64_t(alpha_word) << 32);
			w1[1] = uint64_t(fbmsk) | (uint64_t(fogcol) << 32);
			memcpy(&prims[n], &w0, 16);
			memcpy(reinterpret_cast<char *>(&prims[n]) + 16, &w1, 16);
		}
		if (sp == pos)
		{
			for (uint32_t i = 0; i < 3; i++)
				copy_vertex(positions[3 * n + i], attributes[3 * n + i], pos[i], attr[i]);
		}
		else
		{
			for (uint32_t i = 0; i < nv; i++)
				copy_vertex(positions[3 * n + i], attributes[3 * n + i], sp[i], sa[i]);
			if (nv == 2)
			{
				positions[3 * n + 2] = {};
				attributes[3 * n + 2] = {};
			}
		}
		primitive_count++;
		// Set after any flush above, which clears it.
		last_para_candidate = para_candidate;
		if (current_is_channel_shuffle)
			instances[current_instance].has_channel_shuffle = true;
		// Everything the primitive depends on is up to date now.
		dirty = 0;
	}

	// triangle_is_parallelogram_candidate (gs/gs_util.cpp:237-305): flat
	// attributes, a right angle at one vertex with axis-aligned legs (the
	// triangle's area equals its box's).  order: the right-angle vertex, then
	// the two diagonal ends, the left one first.
	static bool parallelogram_candidate(const pgs_vertex_position *pos, const pgs_vertex_attribute *attr,
	                                    const int32_t *lo, const int32_t *hi, const PrimReg &prim, uint32_t *order)
	{
		if (prim.enables_aa1())
			return false;
		if (!prim.fst && prim.tme && (attr[0].q != attr[1].q || attr[1].q != attr[2].q))
			return false;
		if (pos[0].z != pos[1].z || pos[1].z != pos[2].z)
			return false;
		if (prim.fge && (attr[0].fog != attr[1].fog || attr[1].fog != attr[2].fog))
			return false;
		if (attr[0].rgba != attr[1].rgba || attr[1].rgba != attr[2].rgba)
			return false;
		const int64_t abx = pos[1].x - pos[0].x, aby = pos[1].y - pos[0].y;
		const int64_t acx = pos[2].x - pos[0].x, acy = pos[2].y - pos[0].y;
		const int64_t bcx = pos[2].x - pos[1].x, bcy = pos[2].y - pos[1].y;
		const int64_t cross = abx * acy - aby * acx;
		if ((cross < 0 ? -cross : cross) != int64_t(hi[0] - lo[0]) * int64_t(hi[1] - lo[1]))
			return false;
		int64_t dot;
		if (abx != 0 && aby != 0)
		{
			order[0] = 2; order[1] = 1; order[2] = 0;
			dot = acx * bcx + acy * bcy;
		}
		else if (acx != 0 && acy != 0)
		{
			order[0] = 1; order[1] = 2; order[2] = 0;
			dot = acx * abx + acy * aby;
		}
		else
		{
			order[0] = 0; order[1] = 1; order[2] = 2;
			dot = acx * abx + acy * aby;
		}
		if (dot != 0)
			return false;
		if (pos[order[1]].x > pos[order[2]].x)
			std::swap(order[1], order[2]);
		return true;
	}

	// triangles_form_parallelogram (gs/gs_util.cpp:307-377): the fourth
	// corner is the previous triangle's right-angle vertex, the diagonal is
	// shared, and the attributes continue the previous triangle's.
	static bool forms_parallelogram(const pgs_vertex_position *pos, const pgs_vertex_attribute *attr,
	                                const uint32_t *order, const pgs_vertex_position *last_pos,
	                                const pgs_vertex_attribute *last_attr, const uint32_t *last_order, const PrimReg &prim)
	{
		const pgs_vertex_position &p0 = pos[order[0]], &p1 = pos[order[1]], &p2 = pos[order[2]];
		const pgs_vertex_position &l0 = last_pos[last_order[0]], &l1 = last_pos[last_order[1]],
		                          &l2 = last_pos[last_order[2]];
		if (p1.x + p2.x - p0.x != l0.x || p1.y + p2.y - p0.y != l0.y || p1.x != l1.x || p1.y != l1.y ||
		    p2.x != l2.x || p2.y != l2.y)
			return false;
		if (pos[0].z != last_pos[0].z)
			return false;
		if (!prim.fst && prim.tme && attr[0].q != last_attr[0].q)
			return false;
		if (prim.fge && attr[0].fog != last_attr[0].fog)
			return false;
		if (attr[0].rgba != last_attr[0].rgba)
			return false;
		const pgs_vertex_attribute &a0 = attr[order[0]], &a1 = attr[order[1]], &a2 = attr[order[2]];
		const pgs_vertex_attribute &b0 = last_attr[last_order[0]], &b1 = last_attr[last_order[1]],
		                           &b2 = last_attr[last_order[2]];
		if (prim.tme)
		{
			if (prim.fst)
			{
				const uint16_t u3 = uint16_t(a1.u + a2.u - a0.u), v3 = uint16_t(a1.v + a2.v - a0.v);
				if (u3 != b0.u || v3 != b0.v || a1.u != b1.u || a1.v != b1.v || a2.u != b2.u || a2.v != b2.v)
					return false;
			}
			else
			{
				// Within 1e-4 after the divide by Q: under a sub-texel at 1k x 1k.
				const float es = std::fabs((((a2.s + a1.s) - a0.s) - b0.s) / a0.q);
				const float et = std::fabs((((a2.t + a1.t) - a0.t) - b0.t) / a0.q);
				if (a1.s != b1.s || a1.t != b1.t || a2.s != b2.s || a2.t != b2.t || es > 1e-4f || et > 1e-4f)
					return false;
			}
		}
		return true;
	}

	// ---------------------------------------------------------------
	// GIF packet decode (gs/gs_interface.cpp:4290-4397).
	template <class Sink>
	__attribute__((always_inline)) inline void packed_write(Sink &s, uint32_t desc, const uint64_t *q)
	{
		uint64_t lo = q[0], hi = q[1];
		switch (desc)
		{
		case 0x0: assemble_register(s, R_PRIM, lo & 0x7ff); break;
		case 0x1:
		{
			uint32_t qbits;
			memcpy(&qbits, &dec.internal_q, 4);
			uint64_t v = field(lo, 0, 8) | (uint64_t(field(lo, 32, 8)) << 8) |
			             (uint64_t(field(hi, 0, 8)) << 16) | (uint64_t(field(hi, 32, 8)) << 24) |
			             (uint64_t(qbits) << 32);
			dec.rgbaq = v;
			break;
		}
		case 0x2:
		{
			dec.st = lo;
			uint32_t qbits = uint32_t(hi);
			memcpy(&dec.internal_q, &qbits, 4);
			break;
		}
		case 0x3: dec.uv = field(lo, 0, 14) | (uint64_t(field(lo, 32, 14)) << 16); break;
		case 0x4:
		{
			uint64_t v = field(lo, 0, 16) | (uint64_t(field(lo, 32, 16)) << 16) |
			             (uint64_t(field(hi, 4, 24)) << 32) | (uint64_t(field(hi, 36, 8)) << 56);
			bool adc = field(hi, 47, 1) != 0;
			vertex_kick_xyzf(v);
			drawing_kick(s, adc);
			break;
		}
		case 0x5:
		{
			uint64_t v = field(lo, 0, 16) | (uint64_t(field(lo, 32, 16)) << 16) | (uint64_t(uint32_t(hi)) << 32);
			bool adc = field(hi, 47, 1) != 0;
			vertex_kick_xyz(v);
			drawing_kick(s, adc);
			break;
		}
		case 0xa: dec.fog = uint64_t(field(hi, 36, 8)) << 56; break;
		case 0xc:
		{
			uint64_t v = field(lo, 0, 16) | (uint64_t(field(lo, 32, 16)) << 16) |
			             (uint64_t(field(hi, 4, 24)) << 32) | (uint64_t(field(hi, 36, 8)) << 56);
			vertex_kick_xyzf(v);
			drawing_kick(s, true);
			break;
		}
		case 0xd:
		{
			uint64_t v = field(lo, 0, 16) | (uint64_t(field(lo, 32, 16)) << 16) | (uint64_t(uint32_t(hi)) << 32);
			vertex_kick_xyz(v);
			drawing_kick(s, true);
			break;
		}
		case 0xe: assemble_register(s, uint32_t(hi & 0x7f), lo); break;
		case 0x6: case 0x7: case 0x8: case 0x9: assemble_register(s, desc, lo); break;
		default: break;
		}
	}

	// Whole loops of a register list known at compile time: each write is
	// the one case of packed_write, with no dispatch on the descriptor.
	template <class Sink, uint32_t... D>
	__attribute__((always_inline)) inline void packed_loops(Sink &s, const uint64_t *q, size_t loops)
	{
		constexpr uint32_t nreg = sizeof...(D);
		for (size_t l = 0; l < loops; l++, q += 2 * nreg)
		{
			const uint64_t *w = q;
			((packed_write(s, D, w), w += 2), ...);
		}
	}

	template <class Sink>
	void decode(Sink &s, uint32_t pi, const uint64_t *words, size_t qwords)
	{
		auto &path = dec.paths[pi & 3];
		size_t i = 0;
		while (i < qwords)
		{
			if (path.loop == path.nloop)
			{
				path.tag_lo = words[2 * i];
				path.tag_hi = words[2 * i + 1];
				path.nloop = field(path.tag_lo, 0, 15);
				path.flg = field(path.tag_lo, 58, 2);
				path.nreg = field(path.tag_lo, 60, 4);
				if (path.nreg == 0)
					path.nreg = 16;
				bool pre = field(path.tag_lo, 46, 1) != 0;
				if (path.flg == 0 && pre && path.nloop)
				{
					// GIFtag PRIM field: behaves like an A+D PRIM write.
					assemble_register(s, R_PRIM, field(path.tag_lo, 47, 11));
				}
				path.loop = 0;
				path.reg = 0;
				if (path.nloop)
					dec.internal_q = 1.0f;
				i++;
				continue;
			}

			if (path.flg == 0)
			{
				if (path.reg == 0 && qwords - i >= path.nreg)
				{
					// Whole loops at a time: the descriptors come from the tag once.
					// The usual vertex lists (ST / UV, RGBAQ, XYZ2 and RGBAQ,
					// XYZ2) run a loop with the writes spelled out.
					const size_t loops = std::min<size_t>((qwords - i) / path.nreg, path.nloop - path.loop);
					const uint32_t nreg = path.nreg;
					const uint64_t *q = &words[2 * i];
					const uint64_t list = nreg < 16 ? path.tag_hi & ((uint64_t(1) << (4 * nreg)) - 1) : path.tag_hi;
					if (nreg == 3 && list == 0x512)
						packed_loops<Sink, 0x2, 0x1, 0x5>(s, q, loops);
					else if (nreg == 3 && list == 0x513)
						packed_loops<Sink, 0x3, 0x1, 0x5>(s, q, loops);
					else if (nreg == 2 && list == 0x51)
						packed_loops<Sink, 0x1, 0x5>(s, q, loops);
					else
					{
						uint32_t desc[16];
						for (uint32_t r = 0; r < nreg; r++)
							desc[r] = uint32_t(path.tag_hi >> (4 * r)) & 0xf;
						for (size_t l = 0; l < loops; l++, q += 2 * nreg)
							for (uint32_t r = 0; r < nreg; r++)
								packed_write(s, desc[r], q + 2 * r);
					}
					i += loops * nreg;
					path.loop += uint32_t(loops);
					continue;
				}
				uint32_t desc = uint32_t(path.tag_hi >> (4 * path.reg)) & 0xf;
				packed_write(s, desc, &words[2 * i]);
				i++;
				if (++path.reg == path.nreg)
				{
					path.reg = 0;
					path.loop++;
				}
			}
			else if (path.flg == 1)
			{
				for (uint32_t j = 0; j < 2; j++)
				{
					uint32_t desc = uint32_t(path.tag_hi >> (4 * path.reg)) & 0xf;
					uint64_t v = words[2 * i + j];
					reglist_write(s, desc, v);
					if (++path.reg == path.nreg)
					{
						path.reg = 0;
						path.loop++;
						if (path.loop == path.nloop)
							break;
					}
				}
				i++;
			}
			else
			{
				size_t n = std::min<size_t>(qwords - i, path.nloop - path.loop);
				s.hwreg(&words[2 * i], n * 2);
				i += n;
				path.loop += uint32_t(n);
			}
		}
	}

	template <class Sink>
	void reglist_write(Sink &s, uint32_t desc, uint64_t v)
	{
		// REGLIST: descriptors address registers directly; A+D and NOP are ignored.
		if (desc == 0xe || desc == 0xf || desc == 0xb)
			return;
		if (desc == 0x1)
		{
			dec.rgbaq = v;
			return;
		}
		assemble_register(s, desc, v);
	}

	// A+D register write on the vertex side (the a_d_* handlers,
	// gs/gs_interface.cpp:3506-3990): vertex registers and kicks stay here;
	// PRIM, PRMODE, PRMODECONT and XYOFFSET update the decoder's copies and,
	// like every other register, go on to the state side in stream order.
	template <class Sink>
	void assemble_register(Sink &s, uint32_t addr, uint64_t v)
	{
		addr &= 0x7f;
		switch (addr)
		{
		case R_RGBAQ: case R_RGBAQ_UNDOC: dec.rgbaq = v; return;
		case R_ST: dec.st = v; return;
		case R_UV: dec.uv = v; return;
		case R_FOG: dec.fog = v; return;
		case R_XYZF2: vertex_kick_xyzf(v); drawing_kick(s, false); return;
		case R_XYZ2: vertex_kick_xyz(v); drawing_kick(s, false); return;
		case R_XYZF3: vertex_kick_xyzf(v); drawing_kick(s, true); return;
		case R_XYZ3: vertex_kick_xyz(v); drawing_kick(s, true); return;
		case R_PRIM:
			// With PRMODECONT.AC = 0 only the primitive type comes from PRIM.
			dec.prim = field(dec.prmodecont, 0, 1) ? v : (dec.prim & ~7ull) | (v & 7ull);
			dec.vq.count = 0;
			update_offsets();
			break;
		case R_PRMODE:
			if (!field(dec.prmodecont, 0, 1))
			{
				dec.prim = (v & ~7ull) | (dec.prim & 7ull);
				update_offsets();
			}
			break;
		case R_PRMODECONT: dec.prmodecont = v; break;
		case R_XYOFFSET_1: case R_XYOFFSET_2:
			dec.xyoffset[addr - R_XYOFFSET_1] = v;
			update_offsets();
			break;
		default: break;
		}
		s.reg(addr, v);
		// A host callback sees the stream stopped at its register, as the
		// callback may call back in.
		if ((addr == R_SIGNAL && signal_iface.on_signal) || (addr == R_FINISH && signal_iface.on_finish) ||
		    (addr == R_LABEL && signal_iface.on_label))
			s.barrier();
	}

	// ---------------------------------------------------------------
	// Where the decoder's output goes.  A primitive's vertices are written
	// by the decoder into the slot begin_draw returns.
	struct DrawSlot
	{
		pgs_vertex_position *pos;
		pgs_vertex_attribute *attr;
	};

	// Straight into the state side, on the calling thread.
	struct DirectSink
	{
		explicit DirectSink(pgs_gs *g) : gs(g) {}
		pgs_gs *gs;
		uint32_t nv = 0;
		bool quad = false;
		pgs_vertex_position pos[3];
		pgs_vertex_attribute attr[3];
		void reg(uint32_t addr, uint64_t v) { gs->write_state_register(addr, v); }
		void kick() { gs->post_kick(); }
		void hwreg(const uint64_t *data, size_t count) { gs->hwreg(data, count); }
		DrawSlot begin_draw(uint32_t n, bool q)
		{
			nv = n;
			quad = q;
			return { pos, attr };
		}
		void end_draw() { gs->draw(nv, quad, pos, attr); }
		void barrier() {}
	};

	// Threaded decode.  For large transfers a worker thread runs the decoder
	// over the caller's buffer and hands its output to the calling thread as
	// commands, in chunks through a ring; the calling thread runs the state
	// side (hazards, render passes, the backend, host callbacks) exactly as
	// the direct path does, in stream order, while the worker decodes ahead.
	enum : uint32_t
	{
		CMD_REG = 1, CMD_KICK = 2, CMD_DRAW = 3, CMD_HWREG = 4, CMD_BARRIER = 5, CMD_END = 6,
	};
	static constexpr size_t RING_CHUNK_BYTES = 64 * 1024, RING_CHUNKS = 16;
	static constexpr size_t THREADED_DECODE_MIN_QWORDS = 16 * 1024;
	// How far ahead of the command being run the state side prefetches.
	static constexpr size_t RING_PREFETCH_BYTES = 1024;

	struct CmdRing
	{
		alignas(64) std::atomic<uint64_t> produced{ 0 };
		alignas(64) std::atomic<uint64_t> consumed{ 0 };
		alignas(64) uint32_t used[RING_CHUNKS] = {};
		std::unique_ptr<uint64_t[]> storage{ new uint64_t[RING_CHUNKS * RING_CHUNK_BYTES / 8 + 8] };
		uint8_t *chunk(uint64_t index)
		{
			uint8_t *base = reinterpret_cast<uint8_t *>(storage.get());
			base += (64 - (reinterpret_cast<uintptr_t>(base) & 63)) & 63;
			return base + (index % RING_CHUNKS) * RING_CHUNK_BYTES;
		}
	};

	// Spin on a condition, then yield the core.
	template <class Pred>
	static void wait_until(Pred pred)
	{
		for (uint32_t spins = 0; !pred(); spins++)
			if (spins > 4096)
				std::this_thread::yield();
	}

	// The decoder's side of the ring.  Kicks that draw nothing are counted
	// and handed over with the next command: the state side runs their
	// post_kick calls first.
	struct RingSink
	{
		CmdRing *r;
		uint8_t *cur = nullptr;
		size_t off = 0;
		uint64_t index = 0;
		uint32_t kicks = 0;

		__attribute__((always_inline)) inline uint8_t *reserve(size_t bytes)
		{
			if (!cur || off + bytes > RING_CHUNK_BYTES)
			{
				publish();
				index = r->produced.load(std::memory_order_relaxed);
				const uint64_t idx = index;
				CmdRing *ring = r;
				wait_until([ring, idx] { return idx - ring->consumed.load(std::memory_order_acquire) < RING_CHUNKS; });
				cur = r->chunk(index);
				off = 0;
			}
			uint8_t *p = cur + off;
			off += bytes;
			return p;
		}
		void publish()
		{
			if (!cur)
				return;
			r->used[index % RING_CHUNKS] = uint32_t(off);
			r->produced.store(index + 1, std::memory_order_release);
			cur = nullptr;
		}
		void header(uint8_t *p, uint32_t h) { memcpy(p, &h, 4); }
		void flush_kicks()
		{
			if (kicks)
			{
				header(reserve(8), CMD_KICK | (kicks << 24));
				kicks = 0;
			}
		}
		void reg(uint32_t addr, uint64_t v)
		{
			flush_kicks();
			uint8_t *p = reserve(16);
			header(p, CMD_REG | (addr << 8));
			memcpy(p + 8, &v, 8);
		}
		void kick()
		{
			if (++kicks == 255)
				flush_kicks();
		}
		void hwreg(const uint64_t *data, size_t count)
		{
			flush_kicks();
			uint8_t *p = reserve(24);
			header(p, CMD_HWREG);
			memcpy(p + 8, &data, sizeof(data));
			uint64_t n = count;
			memcpy(p + 16, &n, 8);
		}
		__attribute__((always_inline)) inline DrawSlot begin_draw(uint32_t nv, bool quad)
		{
			uint8_t *p = reserve(8 + 40 * nv);
			header(p, CMD_DRAW | (nv << 8) | (uint32_t(quad) << 16) | (kicks << 24));
			kicks = 0;
			return { reinterpret_cast<pgs_vertex_position *>(p + 8),
			         reinterpret_cast<pgs_vertex_attribute *>(p + 8 + 16 * nv) };
		}
		void end_draw() {}
		// Hands everything over and waits until the state side has run it.
		void barrier()
		{
			flush_kicks();
			header(reserve(8), CMD_BARRIER);
			publish();
			CmdRing *ring = r;
			const uint64_t done = r->produced.load(std::memory_order_relaxed);
			wait_until([ring, done] { return ring->consumed.load(std::memory_order_acquire) == done; });
		}
		void end()
		{
			flush_kicks();
			header(reserve(8), CMD_END);
			publish();
		}
	};

	struct DecodeWorker
	{
		std::thread thread;
		std::mutex mutex;
		std::condition_variable cv;
		uint64_t job_seq = 0;
		std::atomic<uint64_t> done_seq{ 0 };
		bool quit = false;
		uint32_t path = 0;
		const uint64_t *words = nullptr;
		size_t qwords = 0;
		CmdRing ring;
		pid_t pid = 0;
	};
	DecodeWorker *worker = nullptr;
	// pgs_gs_options.threaded_decode.
	uint32_t threaded_decode = 0;

	void worker_main(DecodeWorker *w)
	{
		uint64_t seen = 0;
		for (;;)
		{
			uint32_t pi;
			const uint64_t *words;
			size_t qwords;
			{
				std::unique_lock<std::mutex> lock(w->mutex);
				w->cv.wait(lock, [w, seen] { return w->quit || w->job_seq != seen; });
				if (w->quit)
					return;
				seen = w->job_seq;
				pi = w->path;
				words = w->words;
				qwords = w->qwords;
			}
			RingSink sink{ &w->ring };
			decode(sink, pi, words, qwords);
			sink.end();
			w->done_seq.store(seen, std::memory_order_release);
		}
	}

	void stop_worker()
	{
		if (!worker)
			return;
		if (worker->pid != getpid())
		{
			// A forked child: the thread is not there to join.
			worker = nullptr;
			return;
		}
		{
			std::lock_guard<std::mutex> lock(worker->mutex);
			worker->quit = true;
		}
		worker->cv.notify_one();
		worker->thread.join();
		delete worker;
		worker = nullptr;
	}

	// Runs the state side over the worker's commands until the transfer's end.
	void run_commands(CmdRing &r)
	{
		uint64_t idx = r.consumed.load(std::memory_order_relaxed);
		for (;;)
		{
			const uint64_t want = idx;
			wait_until([&r, want] { return r.produced.load(std::memory_order_acquire) != want; });
			const uint8_t *c = r.chunk(idx);
			const size_t used = r.used[idx % RING_CHUNKS];
			bool end = false;
			for (size_t off = 0; off < used;)
			{
				// The worker wrote this chunk from another core: fetch ahead so
				// the vertex records arrive before draw() reads them.  A draw
				// record spans two lines or more, so two lines per command.
				__builtin_prefetch(c + off + RING_PREFETCH_BYTES, 0, 3);
				__builtin_prefetch(c + off + RING_PREFETCH_BYTES + 64, 0, 3);
				uint32_t h;
				memcpy(&h, c + off, 4);
				switch (h & 0xffu)
				{
				case CMD_REG:
				{
					uint64_t v;
					memcpy(&v, c + off + 8, 8);
					write_state_register(h >> 8, v);
					off += 16;
					break;
				}
				case CMD_KICK:
					for (uint32_t k = h >> 24; k; k--)
						post_kick();
					off += 8;
					break;
				case CMD_DRAW:
				{
					for (uint32_t k = h >> 24; k; k--)
						post_kick();
					const uint32_t nv = (h >> 8) & 0xffu;
					draw(nv, ((h >> 16) & 1u) != 0, reinterpret_cast<const pgs_vertex_position *>(c + off + 8),
					     reinterpret_cast<const pgs_vertex_attribute *>(c + off + 8 + 16 * nv));
					off += 8 + 40 * nv;
					break;
				}
				case CMD_HWREG:
				{
					const uint64_t *data;
					uint64_t n;
					memcpy(&data, c + off + 8, sizeof(data));
					memcpy(&n, c + off + 16, 8);
					hwreg(data, size_t(n));
					off += 24;
					break;
				}
				case CMD_BARRIER:
					off += 8;
					break;
				default:
					end = true;
					off = used;
					break;
				}
			}
			idx++;
			r.consumed.store(idx, std::memory_order_release);
			if (end)
				return;
		}
	}

	bool threaded_transfer(uint32_t pi, const uint64_t *words, size_t qwords)
	{
		if (worker && worker->pid != getpid())
			stop_worker();
		if (!worker)
		{
			auto *w = new (std::nothrow) DecodeWorker();
			if (!w)
				return false;
			w->pid = getpid();
			try
			{
				w->thread = std::thread(&pgs_gs::worker_main, this, w);
			}
			catch (...)
			{
				delete w;
				return false;
			}
			worker = w;
		}
		uint64_t seq;
		{
			std::lock_guard<std::mutex> lock(worker->mutex);
			worker->path = pi;
			worker->words = words;
			worker->qwords = qwords;
			seq = ++worker->job_seq;
		}
		worker->cv.notify_one();
		run_commands(worker->ring);
		DecodeWorker *w = worker;
		wait_until([w, seq] { return w->done_seq.load(std::memory_order_acquire) == seq; });
		return true;
	}

	// GIFInterface::gif_transfer.
	void gif_transfer(uint32_t pi, const uint64_t *words, size_t qwords)
	{
		const bool threaded =
		    threaded_decode == PGS_THREADED_DECODE_ALWAYS ||
		    (threaded_decode == PGS_THREADED_DECODE_AUTO && qwords >= THREADED_DECODE_MIN_QWORDS);
		if (!threaded || !threaded_transfer(pi, words, qwords))
		{
			DirectSink sink(this);
			decode(sink, pi, words, qwords);
		}
		decoder_store();
	}

	// GSInterface::write_register from the host.
	void write_register(uint32_t addr, uint64_t v)
	{
		DirectSink sink(this);
		assemble_register(sink, addr, v);
		decoder_store();
	}

	~pgs_gs() { stop_worker(); }
};

// ---------------------------------------------------------------------------
// C ABI
// ---------------------------------------------------------------------------
extern "C" {

pgs_gs *pgs_gs_create(const pgs_backend_ops *ops, void *backend, const pgs_gs_options *options, int *status)
{
	int dummy;
	if (!status)
		status = &dummy;
	if (!ops || !backend || ops->abi_version < 1 || ops->abi_version > PGS_ABI_VERSION)
	{
		*status = PGS_ERROR_INVALID_ARGUMENT;
		return nullptr;
	}
	if (options && options->struct_size && options->struct_size < offsetof(pgs_gs_options, vram_size) + 4)
	{
		*status = PGS_ERROR_INVALID_ARGUMENT;
		return nullptr;
	}
	if (options && options->vram_size && options->vram_size != PGS_VRAM_SIZE)
	{
		*status = PGS_ERROR_UNSUPPORTED;
		return nullptr;
	}
	auto *gs = new (std::nothrow) pgs_gs();
	if (!gs)
	{
		*status = PGS_ERROR_OUT_OF_MEMORY;
		return nullptr;
	}
	gs->ops = ops;
	gs->be = backend;
	// Power-on register file is all zero, PRMODECONT.AC included
	// (reset_context_state_registers, gs/gs_interface.cpp:32-38).
	// Power-on state: instance 0 does not match any real FRAME/ZBUF.
	gs->instances[0].frame = 0x3full << 24;
	gs->instances[0].zbuf = 0x7ull << 24;
	// Fields past struct_size read as zero (callers built against a shorter
	// layout); struct_size 0 means the whole current layout.
	pgs_gs_options o = {};
	if (options)
	{
		size_t n = options->struct_size ? std::min<size_t>(options->struct_size, sizeof(o)) : sizeof(o);
		memcpy(&o, options, n);
	}
	if (!options)
		o.super_sampling = 1, o.ordered_super_sampling = 1;
	gs->set_super_sampling(o.super_sampling, o.ordered_super_sampling != 0, o.super_sampled_textures != 0);
	if (o.threaded_decode > PGS_THREADED_DECODE_ALWAYS)
	{
		delete gs;
		*status = PGS_ERROR_INVALID_ARGUMENT;
		return nullptr;
	}
	gs->threaded_decode = o.threaded_decode;
	gs->reserve_buffers();
	*status = gs->sticky_error;
	if (gs->sticky_error)
	{
		delete gs;
		return nullptr;
	}
	return gs;
}

void pgs_gs_destroy(pgs_gs *gs)
{
	if (!gs)
		return;
	pgs_gs_dump_close(gs);
	pgs_gs_dump_record_end(gs);
	delete gs;
}

int pgs_gs_gif_transfer(pgs_gs *gs, uint32_t path, const void *data, size_t size)
{
	if (!gs || (size & 15) || path > 3 || (size && !data))
		return PGS_ERROR_INVALID_ARGUMENT;
	if (size == 0)
		return PGS_OK;
	if (gs->dump_out)
		gs->record_transfer(path, data, size);
	gs->gif_transfer(path, static_cast<const uint64_t *>(data), size / 16);
	return gs->sticky_error;
}

int pgs_gs_write_register(pgs_gs *gs, uint32_t addr, uint64_t payload)
{
	if (!gs || addr > 0x7f)
		return PGS_ERROR_INVALID_ARGUMENT;
	if (gs->dump_out)
	{
		// One A+D loop (GSDumpGenerator::write_register): GIF tag NLOOP 1,
		// EOP, PACKED, NREG 1, REGS = A+D; then payload and address.
		const uint64_t words[4] = { 1ull | (1ull << 15) | (1ull << 60), 0xeull, payload, uint64_t(addr) };
		gs->record_transfer(1, words, sizeof(words));
	}
	gs->write_register(addr, payload);
	return gs->sticky_error;
}

int pgs_gs_flush(pgs_gs *gs)
{
	if (!gs)
		return PGS_ERROR_INVALID_ARGUMENT;
	gs->flush();
	return gs->sticky_error;
}

// Whole pages of a host access (map_vram_read / map_vram_write,
// gs/gs_interface.cpp:4184-4255).
static PageRect host_rect(uint64_t offset, uint64_t size)
{
	PageRect r;
	const uint32_t first = uint32_t(offset / PAGE_BYTES), last = uint32_t((offset + size - 1) / PAGE_BYTES);
	r.base_page = first;
	r.page_width = last - first + 1;
	r.page_height = 1;
	r.block_mask = 0xffffffffu;
	r.write_mask = 0xffffffffu;
	return r;
}

// Host reads wait for the work that writes the pages they read.
static void host_read_sync(pgs_gs *gs, uint64_t offset, uint64_t size)
{
	if (size && gs->tracker.host_read_pending(host_rect(offset, size)))
	{
		gs->tracker.mark_submission(PGS_FLUSH_HOST_ACCESS);
		gs->submit();
	}
}

int pgs_gs_read_vram(pgs_gs *gs, uint64_t offset, uint64_t size, void *dst)
{
	if (!gs || !dst || offset + size > PGS_VRAM_SIZE)
		return PGS_ERROR_INVALID_ARGUMENT;
	host_read_sync(gs, offset, size);
	if (gs->sticky_error)
		return gs->sticky_error;
	return gs->ops->read_vram(gs->be, 0, offset, size, dst);
}

int pgs_gs_read_vram_async(pgs_gs *gs, uint64_t offset, uint64_t size, void *dst, uint64_t *ticket)
{
	if (!gs || !dst || !ticket || offset + size > PGS_VRAM_SIZE)
		return PGS_ERROR_INVALID_ARGUMENT;
	host_read_sync(gs, offset, size);
	if (gs->sticky_error)
		return gs->sticky_error;
	if (gs->ops->abi_version >= 2 && gs->ops->read_vram_async && gs->ops->wait_ticket)
		return gs->ops->read_vram_async(gs->be, offset, size, dst, ticket);
	*ticket = 0;
	return gs->ops->read_vram(gs->be, 0, offset, size, dst);
}

int pgs_gs_wait(pgs_gs *gs, uint64_t ticket)
{
	if (!gs)
		return PGS_ERROR_INVALID_ARGUMENT;
	if (ticket == 0)
		return PGS_OK;
	if (gs->ops->abi_version < 2 || !gs->ops->wait_ticket)
		return PGS_ERROR_INVALID_ARGUMENT;
	return gs->ops->wait_ticket(gs->be, ticket);
}

int pgs_gs_write_priv_register(pgs_gs *gs, uint32_t index, uint64_t value)
{
	if (!gs || index >= 15)
		return PGS_ERROR_INVALID_ARGUMENT;
	gs->priv[index] = value;
	return PGS_OK;
}

int pgs_gs_read_priv_register(pgs_gs *gs, uint32_t index, uint64_t *value)
{
	if (!gs || !value || index >= 15)
		return PGS_ERROR_INVALID_ARGUMENT;
	*value = gs->priv[index];
	return PGS_OK;
}

} // extern "C"

namespace
{
// compute_circuit_rect (gs/gs_renderer.cpp:4114-4172) and the sampling
// parameters of sample_crtc_circuit (:4055-4112) for one circuit.  `phase` is
// the field the read-out starts from (alternating-line interlace only).
void circuit_setup(const pgs_gs *gs, uint32_t circuit, uint32_t phase, bool force_progressive, bool high_res,
                   pgs_circuit_params &c, uint32_t &phase_offset)
{
	const uint64_t dispfb = gs->priv[7 + 2 * circuit], display = gs->priv[8 + 2 * circuit];
	const uint64_t smode2 = gs->priv[2];
	bool is_interlaced = field(smode2, 0, 1) != 0;
	bool alternative_sampling = is_interlaced && !field(smode2, 1, 1);
	if (alternative_sampling && force_progressive)
		is_interlaced = false;
	uint32_t DW = field(display, 32, 12) + 1, DH = field(display, 44, 11) + 1;
	uint32_t MAGH = field(display, 23, 4) + 1, MAGV = field(display, 27, 2) + 1;
	uint32_t DY = field(display, 12, 11);
	uint32_t img_w = DW / MAGH, img_h = DH / MAGV, valid_w = img_w, valid_h;
	uint32_t phase_stride = 1;
	phase_offset = 0;
	if (is_interlaced)
	{
		phase_offset = alternative_sampling ? ((DY ^ phase) & 1u) : 0u;
		phase_stride = alternative_sampling ? 2u : 1u;
		valid_h = (img_h - phase_offset + 1) >> 1;
		img_h = (img_h + 1) >> 1;
	}
	else
	{
		valid_h = img_h;
		img_h = (img_h + 1) & ~1u;
	}
	c = {};
	c.fbp = field(dispfb, 0, 9);
	c.fbw = field(dispfb, 9, 6);
	c.psm = field(dispfb, 15, 5);
	c.dbx = field(dispfb, 32, 11);
	c.dby = field(dispfb, 43, 11);
	c.phase = phase_offset;
	c.phase_stride = phase_stride;
	c.super_samples = high_res ? (1u << (gs->sampling_rate_x_log2 + gs->sampling_rate_y_log2)) : 1u;
	uint32_t scale = high_res ? 2u : 1u;
	c.width = img_w * scale;
	c.height = img_h * scale;
	c.valid_width = valid_w * scale;
	c.valid_height = valid_h * scale;
}

// Display mode of SMODE1 (GSRenderer::vsync, gs/gs_renderer.cpp:4262-4378).
struct VideoMode
{
	uint32_t width, height, clock_divider;
	int32_t scan_x, scan_y;
	bool hdtv;
};

bool video_mode(uint64_t smode1, uint64_t smode2, bool overscan, bool tall, VideoMode &m)
{
	enum { CMOD_PROGRESSIVE = 0, CMOD_NTSC = 2, CMOD_PAL = 3 };
	enum { LC_ANALOG = 32, LC_HDTV = 22, LC_VGA = 15, LC_UNKNOWN_29 = 29 };
	const uint32_t cmod = field(smode1, 13, 2), lc = field(smode1, 3, 7);
	const bool interlace = field(smode2, 0, 1) != 0;
	m = {};
	if ((cmod == CMOD_NTSC || (cmod == CMOD_PROGRESSIVE && !interlace)) && lc == LC_ANALOG)
	{
		m = overscan ? VideoMode{ 712, 240, 0, 123, 17, false } : VideoMode{ 640, 224, 0, 159, 25, false };
		m.clock_divider = cmod == CMOD_PROGRESSIVE ? 2u : 4u;
	}
	else if (cmod == CMOD_PAL && lc == LC_ANALOG)
	{
		m = overscan ? VideoMode{ 712, 288, 4, 133, 21, false } : VideoMode{ 640, 256, 4, 169, 36, false };
	}
	else if (cmod == CMOD_PROGRESSIVE && lc == LC_HDTV)
	{
		m = interlace ? VideoMode{ 1920, 540, 1, 236, 0, true } : VideoMode{ 1280, 720, 1, 300, 0, true };
	}
	else if (cmod == CMOD_PROGRESSIVE && lc == LC_VGA)
		return m = VideoMode{ 640, 480, 2, 138, 34, false }, true;
	else if (lc == LC_UNKNOWN_29)
		return m = VideoMode{ 640, 480, 4, 318, 50, false }, true;
	else
		return false;
	if (tall)
	{
		m.height *= 2;
		m.scan_y *= 2;
	}
	return true;
}
} // namespace

extern "C" {

int pgs_gs_scanout_circuit(pgs_gs *gs, uint32_t circuit, uint32_t phase, uint32_t flags, void *dst, uint64_t dst_size,
                           uint32_t *width, uint32_t *height)
{
	if (!gs || circuit > 1 || !width || !height)
		return PGS_ERROR_INVALID_ARGUMENT;
	if (gs->ops->abi_version < 2 || !gs->ops->sample_circuit)
		return PGS_ERROR_UNSUPPORTED;
	gs->flush();
	if (gs->sticky_error)
		return gs->sticky_error;
	const uint64_t smode2 = gs->priv[2], extwrite = gs->priv[13];
	const bool force_progressive = (flags & PGS_SCANOUT_FORCE_PROGRESSIVE) != 0;
	bool alternative_sampling = field(smode2, 0, 1) && !field(smode2, 1, 1);
	// vsync samples the field given by `phase` only for alternating-line
	// interlace that is not forced progressive (:4468-4478).
	uint32_t field_phase = (alternative_sampling && !force_progressive) ? (phase & 1u) : 0u;
	// High-resolution read-out of a super-sampled frame (:4217-4239).
	bool high_res = (flags & PGS_SCANOUT_HIGH_RESOLUTION) != 0;
	if (!force_progressive || field(extwrite, 0, 1) || !gs->sampling_rate_x_log2 || !gs->sampling_rate_y_log2)
		high_res = false;
	pgs_circuit_params c;
	uint32_t phase_offset;
	circuit_setup(gs, circuit, field_phase, force_progressive, high_res, c, phase_offset);
	*width = c.width;
	*height = c.height;
	if (uint64_t(c.width) * c.height * 4u > dst_size || (!dst && c.width && c.height))
		return PGS_ERROR_CAPACITY;
	if (c.width == 0 || c.height == 0)
		return PGS_OK;
	return gs->ops->sample_circuit(gs->be, &c, dst);
}

// GSRenderer::vsync (gs/gs_renderer.cpp:4189-5055): everything that is decided
// from registers happens here; the backend samples, composes, writes back and
// deinterlaces (pgs_merge_params).
static int vsync_scanout(pgs_gs *gs, const pgs_vsync_info *info, uint32_t flags, void *dst, uint64_t dst_size,
                         pgs_scanout_result *res)
{
	*res = {};
	const uint64_t pmode = gs->priv[0], smode1 = gs->priv[1], smode2 = gs->priv[2];
	const uint64_t extbuf = gs->priv[11], extdata = gs->priv[12], extwrite = gs->priv[13], bgcolor = gs->priv[14];
	const bool force_progressive = (flags & PGS_VSYNC_FORCE_PROGRESSIVE) != 0;
	const bool overscan = (flags & PGS_VSYNC_OVERSCAN) != 0;
	const bool crtc_offsets = (flags & PGS_VSYNC_CRTC_OFFSETS) != 0;
	const bool anti_blur = (flags & PGS_VSYNC_ANTI_BLUR) != 0;
	const bool adapt = (flags & PGS_VSYNC_ADAPT_HORIZONTAL) != 0;
	bool high_res = (flags & PGS_VSYNC_HIGH_RESOLUTION) != 0;
	const bool INT = field(smode2, 0, 1) != 0, FFMD = field(smode2, 1, 1) != 0;
	const bool progressive = field(smode1, 13, 2) == 0;
	const bool ext_on = field(extwrite, 0, 1) != 0;
	const uint32_t rx = gs->sampling_rate_x_log2, ry = gs->sampling_rate_y_log2;

	const bool alternative_sampling = INT && !FFMD;
	const bool is_interlaced = INT && !(alternative_sampling && force_progressive);
	const bool force_deinterlace = !high_res && FFMD && INT && !progressive;
	const bool double_strike = !INT && !progressive;
	if (!force_progressive || ext_on || !rx || !ry || force_deinterlace)
		high_res = false;
	bool field_aware = high_res && ry && FFMD && INT && !progressive;

	VideoMode mode;
	if (!video_mode(smode1, smode2, overscan, !is_interlaced && !double_strike && !force_deinterlace, mode))
		return PGS_OK; // unknown video mode: no image
	if (mode.hdtv)
	{
		high_res = false;
		field_aware = false;
	}
	const uint32_t cd = mode.clock_divider;
	const uint32_t phase = (alternative_sampling && !force_progressive) ? (info->phase & 1u) : 0u;

	bool EN1 = field(pmode, 0, 1) != 0, EN2 = field(pmode, 1, 1) != 0;
	uint32_t MMOD = field(pmode, 5, 1), ALP = field(pmode, 8, 8), SLBG = field(pmode, 7, 1);
	if (EN1 && EN2 && anti_blur)
	{
		// Anti-blur: two circuits reading the same buffer one line apart
		// collapse to one (:4478-4531).
		const uint64_t fb1 = gs->priv[7], d1 = gs->priv[8], fb2 = gs->priv[9], d2 = gs->priv[10];
		auto DBY = [](uint64_t fb) { return field(fb, 43, 11); };
		auto DY = [](uint64_t d) { return field(d, 12, 11); };
		auto DX = [](uint64_t d) { return field(d, 0, 12); };
		auto MAGH = [](uint64_t d) { return field(d, 23, 4); };
		if (field(fb1, 0, 9) == field(fb2, 0, 9) && field(fb1, 15, 5) == field(fb2, 15, 5) &&
		    field(fb1, 9, 6) == field(fb2, 9, 6) && field(fb1, 32, 11) == field(fb2, 32, 11) && MAGH(d1) == MAGH(d2) &&
		    field(d1, 27, 2) == field(d2, 27, 2))
		{
			if (MMOD == 1 && DY(d1) == DY(d2) && DBY(fb1) == DBY(fb2) && DX(d1) != DX(d2) &&
			    std::abs(int(DX(d1)) - int(DX(d2))) < int(2 * (MAGH(d1) + 1)))
			{
				EN2 = false;
				ALP = 0xff;
				MMOD = 1;
			}
			else if (alternative_sampling && DY(d1) == DY(d2))
			{
				if (DBY(fb1) + 1 == DBY(fb2))
				{
					EN2 = false;
					ALP = 0xff;
					MMOD = 1;
				}
				else if (DBY(fb1) == DBY(fb2) + 1)
				{
					EN1 = false;
					SLBG = 0;
				}
			}
			else if (alternative_sampling && DBY(fb1) == DBY(fb2))
			{
				if (DY(d1) + 1 == DY(d2))
				{
					EN2 = false;
					ALP = 0xff;
					MMOD = 1;
				}
				else if (DY(d1) == DY(d2) + 1)
				{
					EN1 = false;
					SLBG = 0;
				}
			}
		}
	}

	pgs_merge_params m = {};
	bool has_image[2] = { false, false };
	int32_t shift_x = INT32_MAX, shift_y = INT32_MAX;
	bool skip_shift_x = false, skip_shift_y = false;
	const bool en[2] = { EN1, EN2 };
	for (uint32_t i = 0; i < 2; i++)
	{
		if (!en[i])
			continue;
		const uint64_t display = gs->priv[8 + 2 * i];
		uint32_t phase_offset;
		circuit_setup(gs, i, phase, force_progressive, high_res, m.circuit[i], phase_offset);
		has_image[i] = m.circuit[i].width && m.circuit[i].height;
		if (!has_image[i])
			m.circuit[i] = {};
		int32_t off_x = int32_t(field(display, 0, 12) + cd / 2) / int32_t(cd) - mode.scan_x;
		int32_t off_y = int32_t(field(display, 12, 11) + phase_offset) >> int(is_interlaced);
		off_y -= mode.scan_y;
		uint32_t w = (field(display, 32, 12) + 1) / cd;
		uint32_t h = (field(display, 44, 11) + 1 + uint32_t(is_interlaced)) >> int(is_interlaced);
		if (!is_interlaced)
			h = (h + 1) & ~1u;
		m.rect_x[i] = off_x;
		m.rect_y[i] = off_y;
		m.rect_w[i] = w;
		m.rect_h[i] = h;
		skip_shift_x = skip_shift_x || w != mode.width;
		skip_shift_y = skip_shift_y || h != mode.height;
		shift_x = std::min(shift_x, off_x);
		shift_y = std::min(shift_y, off_y);
	}
	if (!overscan && !crtc_offsets)
	{
		for (uint32_t i = 0; i < 2; i++)
		{
			if (!en[i])
				continue;
			if (!skip_shift_x)
				m.rect_x[i] -= shift_x;
			if (!skip_shift_y)
				m.rect_y[i] -= shift_y;
		}
	}

	const uint32_t real_mode_width = mode.width;
	uint32_t mode_width = mode.width;
	float sampling_rate_mhz = 54.0f / float(cd);
	if (cd == 4 && !is_interlaced)
		sampling_rate_mhz *= 2.0f;
	if (adapt)
	{
		// Express the CRTC rectangles in the circuits' own horizontal resolution
		// (:4646-4685).
		const uint32_t hr_scale = high_res ? 1u : 0u;
		uint32_t h0 = has_image[0] ? (m.circuit[0].width >> hr_scale) : 0u;
		uint32_t h1 = has_image[1] ? (m.circuit[1].width >> hr_scale) : 0u;
		uint32_t magh1 = field(gs->priv[8], 23, 4) + 1, magh2 = field(gs->priv[10], 23, 4) + 1;
		if (h0 == 0)
		{
			h0 = h1;
			magh1 = magh2;
		}
		if (h1 == 0)
			h1 = h0;
		if (h0 && h0 == h1)
		{
			float scaling = float(cd) / float(magh1);
			sampling_rate_mhz *= scaling;
			for (uint32_t i = 0; i < 2; i++)
			{
				if (!en[i])
					continue;
				m.rect_x[i] = int32_t(std::round(float(m.rect_x[i]) * scaling));
				m.rect_w[i] = uint32_t(std::round(float(m.rect_w[i]) * scaling));
			}
			mode_width = uint32_t(std::round(float(mode_width) * scaling));
		}
	}

	res->mode_width = mode_width;
	res->mode_height = mode.height;
	res->high_resolution_scanout = high_res;
	res->sampling_rate_mhz = sampling_rate_mhz;
	res->double_strike = double_strike;

	if ((flags & PGS_VSYNC_RAW_CIRCUIT) && !crtc_offsets && !overscan && adapt && !force_deinterlace &&
	    !is_interlaced && !ext_on)
	{
		// A single unblended circuit that fits the mode goes out as it is (:4695-4735).
		const uint32_t ew = mode_width << int(high_res), eh = mode.height << int(high_res);
		bool raw1 = has_image[0] && !has_image[1] && MMOD == 1 && ALP == 0xff && m.circuit[0].width <= ew &&
		            m.circuit[0].height <= eh;
		bool raw2 = has_image[1] && !has_image[0] && SLBG == 0 && m.circuit[1].width <= ew &&
		            m.circuit[1].height <= eh;
		if (raw1 || raw2)
		{
			const pgs_circuit_params &c = m.circuit[raw1 ? 0 : 1];
			m.raw_circuit = raw1 ? 1u : 2u;
			res->width = c.width;
			res->height = c.height;
			res->internal_width = c.width >> int(high_res);
			res->internal_height = c.height >> int(high_res);
			if (uint64_t(c.width) * c.height * 4u > dst_size || !dst)
				return PGS_ERROR_CAPACITY;
			return gs->ops->vsync(gs->be, &m, dst);
		}
	}

	res->internal_width = mode_width;
	res->internal_height = mode.height;
	m.width = mode_width << int(high_res);
	m.height = mode.height << int(high_res);
	if (field_aware)
		m.height--;
	for (uint32_t i = 0; i < 2; i++)
	{
		if (high_res)
		{
			m.rect_x[i] *= 2;
			m.rect_y[i] *= 2;
			m.rect_w[i] *= 2;
			m.rect_h[i] *= 2;
			if (field_aware && !info->phase)
				m.rect_y[i] -= 1;
		}
	}
	m.draw_circuit2 = SLBG == 0 && has_image[1];
	m.draw_circuit1 = has_image[0];
	m.blend = MMOD == 1 ? (ALP != 0xff ? 1u : 0u) : 2u;
	m.alp = ALP;
	m.bgcolor = uint32_t(bgcolor & 0xffffffu);

	if (ext_on)
	{
		// EXTWRITE feedback (:4900-4990).
		uint32_t rw = field(extdata, 32, 12) + 1, rh = field(extdata, 44, 11) + 1;
		if (!field(extbuf, 22, 1))
			rh *= 2;
		const uint32_t fbin = field(extbuf, 20, 2);
		m.ext_source = fbin == 0 ? 0u : (has_image[1] ? 1u : (has_image[0] ? 2u : 3u));
		if (m.ext_source != 3u)
		{
			const uint32_t smph = field(extdata, 23, 4), smpv = field(extdata, 27, 2);
			const uint32_t scan_w = real_mode_width, scan_h = m.height;
			rw = std::min<uint32_t>(rw, (scan_w * cd + smph) / (smph + 1));
			rh = std::min<uint32_t>(rh, (scan_h + smpv) / (smpv + 1));
			m.ext_write = rw && rh;
			m.ext_width = rw;
			m.ext_height = rh;
			m.ext_wdx = field(extbuf, 32, 11);
			m.ext_wdy = field(extbuf, 43, 11);
			m.ext_exbp = field(extbuf, 0, 14);
			m.ext_exbw = field(extbuf, 14, 6);
			m.ext_emoda = field(extbuf, 23, 2);
			m.ext_emodc = field(extbuf, 25, 2);
			m.ext_uv_base[0] = 0.5f / float(rw);
			m.ext_uv_base[1] = 0.5f / float(rh);
			m.ext_uv_scale[0] = float(smph + 1) / float(scan_w * cd);
			m.ext_uv_scale[1] = float(smpv + 1) / float(scan_h);
		}
		else
			m.ext_source = 0;
	}

	const bool should_deinterlace = !high_res && (is_interlaced || force_deinterlace);
	m.deinterlace = should_deinterlace && !(flags & PGS_VSYNC_SKIP_DEINTERLACE);
	m.phase = info->phase & 1u;
	res->interlaced = should_deinterlace;
	res->interlace_phase = info->phase;
	res->width = m.width;
	res->height = m.deinterlace ? 2 * m.height : m.height;
	if (uint64_t(res->width) * res->height * 4u > dst_size || (!dst && res->width && res->height))
		return PGS_ERROR_CAPACITY;
	return gs->ops->vsync(gs->be, &m, dst);
}

int pgs_gs_write_vram(pgs_gs *gs, uint64_t offset, uint64_t size, const void *src)
{
	if (!gs || !src || offset + size > PGS_VRAM_SIZE)
		return PGS_ERROR_INVALID_ARGUMENT;
	if (!size)
		return PGS_OK;
	const PageRect r = host_rect(offset, size);
	// Work that still reads or writes these pages goes first.
	if (gs->tracker.host_write_pending(r))
	{
		gs->tracker.mark_submission(PGS_FLUSH_HOST_ACCESS);
		gs->submit();
	}
	// Textures of the open pass are decoded when it begins.
	gs->protect_pass_textures(r, PGS_FLUSH_HOST_ACCESS);
	int st = gs->ops->write_vram(gs->be, offset, size, src);
	// The host write replaces these pages (commit_host_write,
	// gs/page_tracker.cpp:700-715).
	gs->tracker.commit_host_write(r);
	return st;
}

int pgs_gs_read_transfer_fifo(pgs_gs *gs, void *data, uint32_t num_128b_words)
{
	if (!gs || (!data && num_128b_words))
		return PGS_ERROR_INVALID_ARGUMENT;
	auto &x = gs->xfer;
	uint32_t avail = x.fifo_size > x.fifo_offset ? x.fifo_size - x.fifo_offset : 0;
	uint32_t n = std::min(avail, num_128b_words);
	if (n)
		memcpy(data, x.fifo.data() + 16ull * x.fifo_offset, 16ull * n);
	if (n < num_128b_words)
		memset(static_cast<uint8_t *>(data) + 16ull * n, 0, 16ull * (num_128b_words - n));
	x.fifo_offset += n;
	return PGS_OK;
}

int pgs_gs_consume_flush_stats(pgs_gs *gs, pgs_flush_stats *stats)
{
	if (!gs || !stats)
		return PGS_ERROR_INVALID_ARGUMENT;
	*stats = gs->stats;
	gs->stats = {};
	return PGS_OK;
}

int pgs_gs_set_super_sampling_rate(pgs_gs *gs, uint32_t super_sampling, uint32_t ordered_grid)
{
	if (!gs)
		return PGS_ERROR_INVALID_ARGUMENT;
	gs->flush();
	gs->set_super_sampling(super_sampling, ordered_grid != 0, gs->ssaa_textures);
	return gs->sticky_error;
}

int pgs_gs_set_super_sampled_textures(pgs_gs *gs, int enable)
{
	if (!gs)
		return PGS_ERROR_INVALID_ARGUMENT;
	gs->flush();
	// Super-sampled textures need a super-sampled frame (set_super_sampling_rate
	// turns them off at X1, gs/gs_interface.cpp:74-78).
	gs->ssaa_textures = enable != 0 && (gs->sampling_rate_x_log2 | gs->sampling_rate_y_log2) != 0;
	gs->reg_serial++;
	gs->template_dirty = true;
	return gs->sticky_error;
}

int pgs_gs_vsync(pgs_gs *gs, const pgs_vsync_info *info, void *dst, uint64_t dst_size, pgs_scanout_result *res)
{
	if (!gs || !info || !res)
		return PGS_ERROR_INVALID_ARGUMENT;
	if (gs->ops->abi_version < 3 || !gs->ops->vsync)
		return PGS_ERROR_UNSUPPORTED;
	gs->flush();
	if (gs->sticky_error)
		return gs->sticky_error;

	// GSInterface::vsync (gs/gs_interface.cpp:4626-4690): a recent tall
	// SCANMSK primitive turns progressive read-out off, and field-aware
	// rendering is chosen for the primitives drawn after this vsync.
	uint32_t flags = info->flags;
	if (gs->complex_scanmsk_timeout)
		flags &= ~PGS_VSYNC_FORCE_PROGRESSIVE;
	const uint64_t smode1 = gs->priv[1], smode2 = gs->priv[2];
	const bool field_aware = (info->flags & PGS_VSYNC_HIGH_RESOLUTION) && gs->sampling_rate_y_log2 &&
	                         field(smode2, 1, 1) && field(smode2, 0, 1) && field(smode1, 13, 2) != 0;
	if (field_aware != gs->field_aware)
	{
		gs->field_aware = field_aware;
		gs->reg_serial++;
		gs->template_dirty = true;
	}

	int r = vsync_scanout(gs, info, flags, dst, dst_size, res);
	if (r != PGS_ERROR_CAPACITY && gs->complex_scanmsk_timeout)
		gs->complex_scanmsk_timeout--;
	return r;
}

int pgs_gs_vsync_can_skip(const pgs_gs *gs, const pgs_vsync_info *info)
{
	if (!gs || !info)
		return PGS_ERROR_INVALID_ARGUMENT;
	// GSRenderer::scanout_is_interlaced (gs/gs_renderer.cpp:4174-4187).
	const uint64_t smode2 = gs->priv[2];
	const bool INT = field(smode2, 0, 1) != 0, FFMD = field(smode2, 1, 1) != 0;
	bool interlaced = INT;
	if (INT && !FFMD && (info->flags & PGS_VSYNC_FORCE_PROGRESSIVE))
		interlaced = false;
	return (gs->complex_scanmsk_timeout == 0 && !interlaced) ? 1 : 0;
}

int pgs_gs_set_hacks(pgs_gs *gs, const pgs_hacks *hacks)
{
	if (!gs || !hacks)
		return PGS_ERROR_INVALID_ARGUMENT;
	if (hacks->backbuffer_promotion)
		return PGS_ERROR_UNSUPPORTED;
	gs->flush();
	gs->hack_disable_mipmaps = hacks->disable_mipmaps != 0;
	gs->hack_unsynced_readbacks = hacks->unsynced_readbacks != 0;
	gs->hack_blend_demote = hacks->allow_blend_demote != 0;
	gs->reg_serial++;
	gs->template_dirty = true;
	return gs->sticky_error;
}

int pgs_gs_reset_context_state(pgs_gs *gs)
{
	if (!gs)
		return PGS_ERROR_INVALID_ARGUMENT;
	gs->flush();
	memset(gs->regs, 0, sizeof(gs->regs));
	for (auto &p : gs->dec.paths)
		p = pgs_gs::Path();
	gs->dec.internal_q = 1.0f;
	gs->clobber_state();
	return gs->sticky_error;
}

int pgs_gs_clobber_register_state(pgs_gs *gs)
{
	if (!gs)
		return PGS_ERROR_INVALID_ARGUMENT;
	gs->clobber_state();
	return PGS_OK;
}

int pgs_gs_read_register(const pgs_gs *gs, uint32_t addr, uint64_t *value)
{
	if (!gs || !value || addr >= 128)
		return PGS_ERROR_INVALID_ARGUMENT;
	*value = gs->read_reg(addr);
	return PGS_OK;
}

int pgs_gs_set_register(pgs_gs *gs, uint32_t addr, uint64_t value)
{
	if (!gs || addr >= 128)
		return PGS_ERROR_INVALID_ARGUMENT;
	gs->set_reg(addr, value);
	return PGS_OK;
}

int pgs_gs_get_gif_path(const pgs_gs *gs, uint32_t path, pgs_gif_path *out)
{
	if (!gs || !out || path >= 4)
		return PGS_ERROR_INVALID_ARGUMENT;
	const auto &p = gs->dec.paths[path];
	out->tag[0] = p.tag_lo;
	out->tag[1] = p.tag_hi;
	out->reg = p.reg;
	out->loop = p.loop;
	return PGS_OK;
}

int pgs_gs_set_gif_path(pgs_gs *gs, uint32_t path, const pgs_gif_path *in)
{
	if (!gs || !in || path >= 4)
		return PGS_ERROR_INVALID_ARGUMENT;
	pgs_gs::Path p;
	p.tag_lo = in->tag[0];
	p.tag_hi = in->tag[1];
	p.nloop = field(p.tag_lo, 0, 15);
	p.flg = field(p.tag_lo, 58, 2);
	p.nreg = field(p.tag_lo, 60, 4);
	if (p.nreg == 0)
		p.nreg = 16;
	if (in->loop > p.nloop || in->reg >= p.nreg)
		return PGS_ERROR_INVALID_ARGUMENT;
	p.reg = in->reg;
	p.loop = in->loop;
	gs->dec.paths[path] = p;
	return PGS_OK;
}

int pgs_gs_set_signal_interface(pgs_gs *gs, const pgs_signal_interface *iface)
{
	if (!gs)
		return PGS_ERROR_INVALID_ARGUMENT;
	gs->signal_iface = iface ? *iface : pgs_signal_interface{};
	return PGS_OK;
}

int pgs_gs_set_debug_mode(pgs_gs *gs, const pgs_debug_mode *mode)
{
	if (!gs || !mode || mode->draw_mode > 2)
		return PGS_ERROR_INVALID_ARGUMENT;
	gs->debug_mode = *mode;
	if (gs->ops->abi_version >= 4 && gs->ops->timestamps)
		return gs->ops->timestamps(gs->be, mode->timestamps ? 1 : 0, nullptr);
	return PGS_OK;
}

int pgs_gs_get_accumulated_timestamps(pgs_gs *gs, uint32_t type, double *seconds)
{
	if (!gs || !seconds || type >= PGS_TIMESTAMP_COUNT)
		return PGS_ERROR_INVALID_ARGUMENT;
	*seconds = 0.0;
	if (gs->ops->abi_version < 4 || !gs->ops->timestamps)
		return PGS_OK;
	double totals[PGS_TIMESTAMP_COUNT] = {};
	int r = gs->ops->timestamps(gs->be, -1, totals);
	if (r == PGS_OK)
		*seconds = totals[type];
	return r;
}
}

// ---------------------------------------------------------------------------
// GS dumps (PCSX2 / GSdx format as read by GSDumpParser, dump/gs_dump_parser.cpp,
// and written by GSDumpGenerator, dump/gs_dump_generator.cpp).
namespace
{
constexpr uint32_t DUMP_STATE_VERSION = 9, DUMP_STATE_VERSION_MIN = 8;
constexpr size_t PRIV_STATE_BYTES = 2 * 0x200 * 8;   // PrivRegisterState: two 0x200-qword halves
enum : uint8_t { DUMP_TRANSFER = 0, DUMP_VSYNC = 1, DUMP_READ_FIFO = 2, DUMP_PRIV = 3 };

// Register file order of the dump's state block (read_register_state).
constexpr uint32_t DUMP_GLOBAL_REGS[] = { R_PRIM, R_PRMODECONT, R_TEXCLUT, R_SCANMSK, R_TEXA, R_FOGCOL, R_DIMX,
                                          R_DTHE, R_COLCLAMP, R_PABE, R_BITBLTBUF, R_TRXDIR, R_TRXPOS, R_TRXREG };
constexpr uint32_t DUMP_CTX_REGS[] = { R_XYOFFSET_1, R_TEX0_1, R_TEX1_1, R_CLAMP_1, R_MIPTBP1_1, R_MIPTBP2_1,
                                       R_SCISSOR_1, R_ALPHA_1, R_TEST_1, R_FBA_1, R_FRAME_1, R_ZBUF_1 };

bool rd(FILE *f, void *p, size_t n) { return fread(p, 1, n, f) == n; }
bool wr(FILE *f, const void *p, size_t n) { return fwrite(p, 1, n, f) == n; }
template <typename T> bool rdv(FILE *f, T &v) { return rd(f, &v, sizeof(v)); }
template <typename T> bool wrv(FILE *f, const T &v) { return wr(f, &v, sizeof(v)); }
}

extern "C" {
int pgs_gs_dump_open(pgs_gs *gs, const char *path)
{
	if (!gs || !path)
		return PGS_ERROR_INVALID_ARGUMENT;
	pgs_gs_dump_close(gs);
	FILE *f = fopen(path, "rb");
	if (!f)
		return PGS_ERROR_IO;
	auto fail = [&]() { fclose(f); return PGS_ERROR_IO; };
	uint32_t crc = 0, header_size = 0, header[9] = {};
	if (!rdv(f, crc) || crc != 0xffffffffu || !rdv(f, header_size) || header_size < sizeof(header) ||
	    !rd(f, header, sizeof(header)) || header[0] < DUMP_STATE_VERSION_MIN || header[0] > DUMP_STATE_VERSION)
		return fail();
	if (fseek(f, long(header_size - sizeof(header)), SEEK_CUR) != 0)
		return fail();
	uint32_t version = 0;
	uint64_t v64 = 0;
	uint32_t v32 = 0;
	if (!rdv(f, version))
		return fail();
	uint64_t regs[128];
	memcpy(regs, gs->regs, sizeof(regs));
	for (uint32_t r : DUMP_GLOBAL_REGS)
		if (!rdv(f, regs[r]))
			return fail();
	if (!rdv(f, v64))   // dummy
		return fail();
	for (uint32_t ctx = 0; ctx < 2; ctx++)
		for (uint32_t r : DUMP_CTX_REGS)
			if (!rdv(f, regs[r + ctx]))
				return fail();
	if (!rdv(f, regs[R_RGBAQ]) || !rdv(f, regs[R_ST]) || !rdv(f, v32))
		return fail();
	regs[R_UV] = v32;
	if (!rdv(f, v32))
		return fail();
	regs[R_FOG] = v32;
	uint8_t skip[8 + 4 * 4 + 61];
	if (!rd(f, skip, 8 + 4 * 4) || (version >= 9 && !rd(f, skip, 61)))
		return fail();
	std::vector<uint8_t> vram(PGS_VRAM_SIZE);
	if (!rd(f, vram.data(), vram.size()))
		return fail();
	uint64_t tags[4][2];
	uint32_t path_reg[4];
	for (int i = 0; i < 4; i++)
		if (!rd(f, tags[i], 16) || !rdv(f, path_reg[i]))
			return fail();
	float q = 1.0f;
	std::vector<uint64_t> priv(PRIV_STATE_BYTES / 8);
	if (!rdv(f, q) || !rd(f, priv.data(), PRIV_STATE_BYTES))
		return fail();

	// Restore: VRAM through the backend, then the register file as-is
	// (clobber_register_state: no side effects, every derived state dirty).
	gs->flush();
	int r = gs->ops->write_vram(gs->be, 0, PGS_VRAM_SIZE, vram.data());
	if (r)
	{
		fclose(f);
		return r;
	}
	memcpy(gs->regs, regs, sizeof(regs));
	gs->dec.internal_q = q;
	for (int i = 0; i < 4; i++)
	{
		auto &p = gs->dec.paths[i];
		p.tag_lo = tags[i][0];
		p.tag_hi = tags[i][1];
		p.nloop = field(p.tag_lo, 0, 15);
		p.flg = field(p.tag_lo, 58, 2);
		p.nreg = field(p.tag_lo, 60, 4);
		if (p.nreg == 0)
			p.nreg = 16;
		p.loop = 0;
		p.reg = path_reg[i];
	}
	for (int i = 0; i < 15; i++)
		gs->priv[i] = priv[2 * i];
	gs->clobber_state();
	gs->write_register(R_TEXFLUSH, 0);
	gs->dump_in = f;
	return gs->sticky_error;
}

int pgs_gs_dump_next_vsync(pgs_gs *gs, uint32_t *field_out)
{
	if (!gs || !gs->dump_in)
		return PGS_ERROR_INVALID_ARGUMENT;
	FILE *f = gs->dump_in;
	bool has_transfer = false;
	for (;;)
	{
		uint8_t type;
		if (!rdv(f, type))
			return 0;
		switch (type)
		{
		case DUMP_TRANSFER:
		{
			uint8_t path;
			uint32_t size;
			if (!rdv(f, path) || !rdv(f, size))
				return 0;
			gs->dump_buf.resize((size + 15) / 8 + 2);
			if (!rd(f, gs->dump_buf.data(), size))
				return 0;
			if (size >= 16)
				gs->gif_transfer(path & 3, gs->dump_buf.data(), size / 16);
			has_transfer = true;
			break;
		}
		case DUMP_VSYNC:
		{
			uint8_t fld;
			if (!rdv(f, fld))
				return 0;
			gs->flush();
			if (has_transfer)
			{
				if (field_out)
					*field_out = fld;
				return gs->sticky_error ? gs->sticky_error : 1;
			}
			break;
		}
		case DUMP_PRIV:
		{
			std::vector<uint64_t> priv(PRIV_STATE_BYTES / 8);
			if (!rd(f, priv.data(), PRIV_STATE_BYTES))
				return 0;
			for (int i = 0; i < 15; i++)
				gs->priv[i] = priv[2 * i];
			break;
		}
		case DUMP_READ_FIFO:
		{
			// As the reference's parser: the FIFO read is not replayed.
			uint32_t size;
			if (!rdv(f, size))
				return 0;
			if (field_out)
				*field_out = 0;
			return 1;
		}
		default:
			return PGS_ERROR_IO;
		}
	}
}

int pgs_gs_dump_close(pgs_gs *gs)
{
	if (!gs)
		return PGS_ERROR_INVALID_ARGUMENT;
	if (gs->dump_in)
		fclose(gs->dump_in);
	gs->dump_in = nullptr;
	return PGS_OK;
}

int pgs_gs_dump_record_begin(pgs_gs *gs, const char *path)
{
	if (!gs || !path)
		return PGS_ERROR_INVALID_ARGUMENT;
	pgs_gs_dump_record_end(gs);
	gs->flush();
	std::vector<uint8_t> vram(PGS_VRAM_SIZE);
	int r = gs->ops->read_vram(gs->be, 0, 0, PGS_VRAM_SIZE, vram.data());
	if (r)
		return r;
	FILE *f = fopen(path, "wb");
	if (!f)
		return PGS_ERROR_IO;
	bool ok = true;
	uint32_t header[9] = {};
	header[0] = DUMP_STATE_VERSION;
	header[1] = uint32_t(PGS_VRAM_SIZE + (18 + 12 * 2) * 8 + 7 * 4 + 4 * 5 * 4 + 4);
	ok = ok && wrv(f, uint32_t(0xffffffffu)) && wrv(f, uint32_t(sizeof(header))) && wr(f, header, sizeof(header));
	ok = ok && wrv(f, DUMP_STATE_VERSION_MIN);
	for (uint32_t reg : DUMP_GLOBAL_REGS)
		ok = ok && wrv(f, gs->regs[reg]);
	ok = ok && wrv(f, gs->regs[R_TRXREG]);   // dummy
	for (uint32_t ctx = 0; ctx < 2; ctx++)
		for (uint32_t reg : DUMP_CTX_REGS)
			ok = ok && wrv(f, gs->regs[reg + ctx]);
	ok = ok && wrv(f, gs->read_reg(R_RGBAQ)) && wrv(f, gs->read_reg(R_ST)) && wrv(f, uint32_t(gs->read_reg(R_UV))) &&
	     wrv(f, uint32_t(gs->read_reg(R_FOG))) && wrv(f, uint64_t(0)) && wrv(f, 0xffffffffu) && wrv(f, 0xffffffffu) &&
	     wrv(f, uint32_t(0)) && wrv(f, uint32_t(0));
	ok = ok && wr(f, vram.data(), vram.size());
	for (int i = 0; i < 4; i++)
	{
		const auto &p = gs->dec.paths[i];
		uint64_t lo = p.tag_lo;
		// NLOOP minus the loops already done (the format has no loop counter).
		uint32_t remaining = p.nloop >= p.loop ? p.nloop - p.loop : 0;
		lo = (lo & ~0x7fffull) | (remaining & 0x7fffu);
		ok = ok && wrv(f, lo) && wrv(f, p.tag_hi) && wrv(f, p.reg);
	}
	ok = ok && wrv(f, gs->dec.internal_q);
	std::vector<uint64_t> priv(PRIV_STATE_BYTES / 8, 0);
	for (int i = 0; i < 15; i++)
		priv[2 * i] = gs->priv[i];
	ok = ok && wr(f, priv.data(), PRIV_STATE_BYTES);
	if (!ok)
	{
		fclose(f);
		return PGS_ERROR_IO;
	}
	gs->dump_out = f;
	return PGS_OK;
}

int pgs_gs_dump_record_vsync(pgs_gs *gs, uint32_t fld)
{
	if (!gs || !gs->dump_out)
		return PGS_ERROR_INVALID_ARGUMENT;
	std::vector<uint64_t> priv(PRIV_STATE_BYTES / 8, 0);
	for (int i = 0; i < 15; i++)
		priv[2 * i] = gs->priv[i];
	bool ok = wrv(gs->dump_out, uint8_t(DUMP_PRIV)) && wr(gs->dump_out, priv.data(), PRIV_STATE_BYTES) &&
	          wrv(gs->dump_out, uint8_t(DUMP_VSYNC)) && wrv(gs->dump_out, uint8_t(fld));
	return ok ? PGS_OK : PGS_ERROR_IO;
}

int pgs_gs_dump_record_end(pgs_gs *gs)
{
	if (!gs)
		return PGS_ERROR_INVALID_ARGUMENT;
	int r = PGS_OK;
	if (gs->dump_out && fclose(gs->dump_out) != 0)
		r = PGS_ERROR_IO;
	gs->dump_out = nullptr;
	return r;
}
}
