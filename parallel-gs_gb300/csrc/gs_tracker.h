// gs_tracker.h -- VRAM hazard tracking of the frontend (host code).
//
// The frontend decides where render passes end from which 256-byte blocks of
// which 8 KiB pages a pass writes as frame or depth buffer, which blocks
// textures, CLUT loads and transfers read and write, and which bits of each
// 32-bit word those accesses touch.  This follows the reference's PageTracker
// (gs/page_tracker.cpp, gs/page_tracker.hpp) rule for rule, because the
// decisions are part of the visible result: at a super-sampling rate every
// coarse tile's sampling decision depends on what shares its pass.  The
// texture cache is modelled only as far as it decides those flushes and the
// validity of the textures a pass already holds (no images are kept: the
// backend decodes the textures of a pass from VRAM as the pass begins).
//
// Page rectangles follow compute_page_rect (gs/gs_util.cpp:141-230) and its
// block masks swizzle_block_mask_PS2 (gs/shaders/swizzle_utils.h:183-302).
#pragma once
#include "gs_defs.h"

#include <cstdint>
#include <cstring>
#include <unordered_map>
#include <vector>

namespace pgs
{
constexpr uint32_t TRACKER_PAGES = VRAM_SIZE / PAGE_BYTES;

struct PageRect
{
	uint32_t base_page = 0, page_width = 0, page_height = 0, page_stride = 0;
	uint32_t block_mask = 0, write_mask = 0;
};

// Bits of a 32-bit word a format stores (psm_word_write_mask, gs/gs_util.cpp:13-29).
inline uint32_t psm_word_write_mask(uint32_t psm)
{
	switch (psm)
	{
	case PSMCT24: case PSMZ24: return 0xffffffu;
	case PSMT8H: return 0xffu << 24;
	case PSMT4HL: return 0xfu << 24;
	case PSMT4HH: return 0xfu << 28;
	default: return 0xffffffffu;
	}
}

// Index of block (bx, by) of a buffer whose base is `base` blocks into a page,
// as the hazard masks number blocks: the 32-bit order for the 32/24-bit colour
// formats and PSMT8 / 8H / 4HL / 4HH, the 16-bit order for PSMCT16 and PSMT4,
// the 16S order, and the depth formats XOR 0x18 after the base is added.  Bit
// 32 and up land in the following page.
inline uint32_t mask_block_index(uint32_t base, uint32_t bx, uint32_t by, uint32_t psm)
{
	switch (psm)
	{
	case PSMZ32: case PSMZ24: return (block_order_32(bx, by) + base) ^ 0x18u;
	case PSMCT16: case PSMT4: return block_order_16(bx, by) + base;
	case PSMZ16: return (block_order_16(bx, by) + base) ^ 0x18u;
	case PSMCT16S: return block_order_16s(bx, by) + base;
	case PSMZ16S: return (block_order_16s(bx, by) + base) ^ 0x18u;
	default: return block_order_32(bx, by) + base;
	}
}

inline uint64_t block_mask_two_pages(uint32_t base, uint32_t bx0, uint32_t by0, uint32_t nbx, uint32_t nby,
                                     uint32_t psm)
{
	uint64_t m = 0;
	for (uint32_t y = 0; y < nby; y++)
		for (uint32_t x = 0; x < nbx; x++)
			m |= 1ull << (mask_block_index(base, bx0 + x, by0 + y, psm) & 63u);
	return m;
}

// Pages (and, for a rectangle inside one page, blocks) a w x h rectangle at
// (x, y) of a buffer at base_256 with row_length_64 touches.
inline PageRect compute_page_rect(uint32_t base_256, uint32_t x, uint32_t y, uint32_t w, uint32_t h,
                                  uint32_t row_length_64, uint32_t psm)
{
	PageRect r;
	if (!w || !h)
		return r;
	const Layout L = psm_layout(psm);
	const uint32_t stride = (psm == PSMT4 || psm == PSMT8) ? (row_length_64 >> 1) : row_length_64;
	r.base_page = base_256 / BLOCKS_PER_PAGE;
	r.page_stride = stride;
	r.write_mask = psm_word_write_mask(psm);
	const uint32_t px = x >> L.pw, py = y >> L.ph;
	r.base_page += px + stride * py;
	x -= px << L.pw;
	y -= py << L.ph;
	// Offsets inside the first page widen the rectangle.
	w += x;
	h += y;
	r.page_width = ((w - 1) >> L.pw) + 1;
	r.page_height = ((h - 1) >> L.ph) + 1;
	const uint32_t block_offset = base_256 % BLOCKS_PER_PAGE;
	const uint32_t max_bx = ((w - 1) >> L.bw) % BLOCKS_PER_PAGE;
	const uint32_t max_by = ((h - 1) >> L.bh) % BLOCKS_PER_PAGE;
	const bool single_page = r.page_width == 1 && r.page_height == 1;
	if (block_offset != 0 || single_page)
	{
		const uint32_t min_bx = x >> L.bw, min_by = y >> L.bh;
		uint64_t m;
		if (max_bx < min_bx || max_by < min_by)
			m = ~0ull; // wide rectangles whose block count wraps: every block, both pages
		else
			m = block_mask_two_pages(block_offset, min_bx, min_by, max_bx - min_bx + 1, max_by - min_by + 1, psm);
		const uint32_t hi = uint32_t(m >> 32), lo = uint32_t(m);
		if (hi == 0)
		{
			if (single_page)
				r.block_mask = lo;
		}
		else if (single_page && lo == 0)
		{
			// Only the following page is touched (depth swizzles can do this).
			r.base_page++;
			r.block_mask = hi;
		}
		else
		{
			// Straddles into the next page on every row.
			r.page_width++;
		}
	}
	if (!r.block_mask)
		r.block_mask = 0xffffffffu;
	return r;
}

// What a tracker event asks the frontend to do (PageTrackerFlushFlags,
// gs/page_tracker.hpp:101-115).
enum TrackerFlush : uint32_t
{
	TRACKER_FLUSH_HOST_VRAM_SYNC = 1u << 0,
	TRACKER_FLUSH_COPY = 1u << 1,
	TRACKER_FLUSH_CACHE = 1u << 2,
	TRACKER_FLUSH_FB = 1u << 3,
	TRACKER_FLUSH_WRITE_BACK = 1u << 4,
	TRACKER_FLUSH_FB_ALL = TRACKER_FLUSH_HOST_VRAM_SYNC | TRACKER_FLUSH_CACHE | TRACKER_FLUSH_COPY | TRACKER_FLUSH_FB,
	TRACKER_FLUSH_COPY_ALL = TRACKER_FLUSH_HOST_VRAM_SYNC | TRACKER_FLUSH_COPY,
	TRACKER_FLUSH_CACHE_ALL = TRACKER_FLUSH_HOST_VRAM_SYNC | TRACKER_FLUSH_COPY | TRACKER_FLUSH_CACHE
};

// The frontend side of the tracker (the callbacks GSInterface gives its
// PageTracker).
struct TrackerClient
{
	virtual void tracker_flush(uint32_t flags, uint32_t reason) = 0;
	// A texture of the cache went stale; `clut`: only its palette did.
	virtual void tracker_invalidate_texture(uint64_t hash, bool clut) = 0;
	virtual void tracker_texture_state_dirty_with_flush() = 0;
	virtual void tracker_forget_memoization() = 0;
	virtual ~TrackerClient() = default;
};

class HazardTracker
{
public:
	enum Status : uint8_t { LIVE, FLOATING, DEAD };

	explicit HazardTracker(TrackerClient &client_) : client(client_) { reset(); }

	void reset()
	{
		memset(pages, 0, sizeof(pages));
		for (auto &l : page_textures)
			l.clear();
		for (auto &l : page_short_textures)
			l.clear();
		textures.clear();
		live.clear();
		palette_textures.clear();
		fb_pages.clear();
		cache_pages.clear();
		copy_pages.clear();
		host_pages.clear();
		short_pages.clear();
		invalidate_pages.clear();
		csa_written = 0;
		fb_lo = UINT32_MAX;
		fb_hi = 0;
		fb_mask = 0;
		pressure = false;
	}

	// ---- framebuffer --------------------------------------------------
	void mark_fb_write(const PageRect &r)
	{
		for_pages(r, [&](uint32_t p) {
			Page &s = pages[p];
			note_fb(p);
			note_host(p);
			s.fb_read |= r.block_mask;
			s.fb_write |= r.block_mask;
			s.host_write_pending |= r.block_mask;
			s.host_read_pending |= r.block_mask;
			s.may_super_sample = true;
			if (s.inv_block == 0)
				invalidate_pages.push_back(uint16_t(p));
			s.inv_block = 0xffffffffu;
			s.inv_write = 0xffffffffu;
			s.pending_fb |= r.write_mask;
		});
		// Range of pages with framebuffer writes, unwrapped (an early-out).
		fb_lo = std::min(fb_lo, r.base_page);
		fb_hi = std::max(fb_hi, r.base_page + (r.page_height - 1) * r.page_stride + r.page_width - 1);
		fb_mask |= r.write_mask;
	}

	void mark_fb_read(const PageRect &r)
	{
		for_pages(r, [&](uint32_t p) {
			Page &s = pages[p];
			note_fb(p);
			note_host(p);
			s.fb_read |= r.block_mask;
			s.host_write_pending |= r.block_mask;
			s.pending_fb |= r.write_mask;
		});
	}

	bool has_fb_write(const PageRect &r) const
	{
		bool hit = false;
		for_pages(r, [&](uint32_t p) {
			const Page &s = pages[p];
			hit = hit || ((s.fb_write & r.block_mask) && (s.pending_fb & r.write_mask));
		});
		return hit;
	}

	bool has_fb_read_write(const PageRect &r) const
	{
		bool hit = false;
		for_pages(r, [&](uint32_t p) {
			const Page &s = pages[p];
			hit = hit || (((s.fb_write | s.fb_read) & r.block_mask) && (s.pending_fb & r.write_mask));
		});
		return hit;
	}

	// Reading a texture or CLUT source: a read after a framebuffer write of
	// the open pass ends it (mark_texture_read, gs/page_tracker.cpp:327-345).
	void mark_texture_read(const PageRect &r)
	{
		if ((r.write_mask & fb_mask) == 0)
			return;
		const uint32_t first = r.base_page, last = r.base_page + (r.page_height - 1) * r.page_stride + r.page_width - 1;
		if (last < fb_lo || first > fb_hi)
			return;
		if (has_fb_write(r))
			flush_render_pass(PGS_FLUSH_TEXTURE_HAZARD);
	}

	bool texture_may_super_sample(const PageRect &r) const
	{
		return pages[r.base_page % TRACKER_PAGES].may_super_sample;
	}

	// ---- transfers ----------------------------------------------------
	// HOST -> LOCAL (mark_transfer_write, gs/page_tracker.cpp:640-686).
	void mark_transfer_write(const PageRect &r)
	{
		bool need_invalidate = false;
		const Blocks b = blocks(r);
		if (has_fb_read_write(r))
			flush_render_pass(PGS_FLUSH_COPY_HAZARD);
		else if (b.cached_read & r.block_mask)
		{
			flush_cached();
			need_invalidate = true;
		}
		else if (b.copy_read & r.block_mask)
			flush_copy();
		for_pages(r, [&](uint32_t p) {
			Page &s = pages[p];
			note_host(p);
			note_copy(p);
			note_invalidate(p);
			s.host_write_pending |= r.block_mask;
			s.host_read_pending |= r.block_mask;
			s.copy_write |= r.block_mask;
			s.inv_block |= r.block_mask;
			s.inv_write |= r.write_mask;
			s.may_super_sample = false;
			if (invalidate(page_short_textures[p], r.block_mask, r.write_mask, UINT32_MAX))
				flush_cached();
		});
		if (need_invalidate)
			invalidate_texture_cache(UINT32_MAX);
	}

	// LOCAL -> LOCAL (mark_transfer_copy, gs/page_tracker.cpp:204-325).
	void mark_transfer_copy(const PageRect &dst, const PageRect &src)
	{
		bool need_invalidate = false;
		const Blocks bd = blocks(dst), bs = blocks(src);
		if (has_fb_read_write(dst) || has_fb_write(src))
			flush_render_pass(PGS_FLUSH_COPY_HAZARD);
		else if (bd.cached_read & dst.block_mask)
		{
			flush_cached();
			need_invalidate = true;
		}
		else if ((bd.copy_read & dst.block_mask) || (bs.copy_write & src.block_mask))
			flush_copy();
		for_pages(dst, [&](uint32_t p) {
			Page &s = pages[p];
			note_host(p);
			note_copy(p);
			note_invalidate(p);
			s.host_write_pending |= dst.block_mask;
			s.host_read_pending |= dst.block_mask;
			s.copy_write |= dst.block_mask;
			s.inv_block |= dst.block_mask;
			s.inv_write |= dst.write_mask;
			s.may_super_sample = false;
			if (invalidate(page_short_textures[p], dst.block_mask, dst.write_mask, UINT32_MAX))
				flush_cached();
		});
		for_pages(src, [&](uint32_t p) {
			Page &s = pages[p];
			note_copy(p);
			note_host(p);
			s.host_write_pending |= dst.block_mask;
			s.copy_read |= src.block_mask;
		});
		if (need_invalidate)
			invalidate_texture_cache(UINT32_MAX);
	}

	// Host writes into VRAM (mark_external_write / commit_host_write,
	// gs/page_tracker.cpp:125-145, 700-715).
	void mark_external_write(const PageRect &r)
	{
		for_pages(r, [&](uint32_t p) {
			Page &s = pages[p];
			note_host(p);
			note_invalidate(p);
			s.host_read_pending |= r.block_mask;
			s.host_write_pending |= r.block_mask;
			s.inv_block |= r.block_mask;
			s.inv_write |= r.block_mask;
			s.may_super_sample = false;
		});
		invalidate_texture_cache(UINT32_MAX);
	}

	// A host write that went straight to VRAM (commit_host_write,
	// gs/page_tracker.cpp:700-715): cached textures of these pages go stale.
	void commit_host_write(const PageRect &r)
	{
		for_pages(r, [&](uint32_t p) {
			Page &s = pages[p];
			s.may_super_sample = false;
			note_invalidate(p);
			s.inv_block = 0xffffffffu;
			s.inv_write = 0xffffffffu;
		});
	}

	// GPU work not yet submitted writes (host_read_pending) or touches
	// (host_write_pending) these blocks: the host must submit and wait before
	// reading / writing them (get_host_read_timeline / get_host_write_timeline
	// returning UINT64_MAX, gs/page_tracker.cpp:36-66, 760-805).  Submitted
	// work counts as complete.
	bool host_read_pending(const PageRect &r) const
	{
		bool pending = false;
		for_pages(r, [&](uint32_t p) { pending = pending || (pages[p].host_read_pending & r.block_mask); });
		return pending;
	}

	bool host_write_pending(const PageRect &r) const
	{
		bool pending = false;
		for_pages(r, [&](uint32_t p) { pending = pending || (pages[p].host_write_pending & r.block_mask); });
		return pending;
	}

	// ---- texture cache --------------------------------------------------
	void register_clut_read(const PageRect &r, uint32_t csa_mask)
	{
		csa_written |= csa_mask;
		for_pages(r, [&](uint32_t p) {
			Page &s = pages[p];
			note_cache(p);
			note_host(p);
			s.host_write_pending |= r.block_mask;
			s.cached_read |= r.block_mask;
		});
	}

	// A cached image of this pass only (register_short_term_cached_texture).
	void register_short_term_texture(const PageRect *levels, uint32_t num_levels, uint64_t hash)
	{
		const uint32_t id = new_texture(hash);
		for (uint32_t l = 0; l < num_levels; l++)
		{
			const PageRect &r = levels[l];
			for_pages(r, [&](uint32_t p) {
				Page &s = pages[p];
				note_host(p);
				note_cache(p);
				s.host_write_pending |= r.block_mask;
				s.cached_read |= r.block_mask;
				collect_dead(page_short_textures[p]);
				if (page_short_textures[p].empty())
					short_pages.push_back(uint16_t(p));
				page_short_textures[p].push_back({ id, r.block_mask, r.write_mask, UINT32_MAX });
			});
		}
	}

	// A long-term cached image (register_cached_texture,
	// gs/page_tracker.cpp:432-495).  Small single-page textures whose pages
	// have no pending GPU writes are read from host memory at once and leave
	// no cached-read marks.
	void register_texture(const PageRect *levels, uint32_t num_levels, uint32_t csa_mask, uint32_t clut_instance,
	                      uint64_t hash)
	{
		const uint32_t id = new_texture(hash);
		live[hash] = id;
		const bool on_cpu = num_levels == 1 && levels[0].page_width == 1 && levels[0].page_height == 1 &&
		                    !host_read_pending(levels[0]);
		for (uint32_t l = 0; l < num_levels; l++)
		{
			const PageRect &r = levels[l];
			for_pages(r, [&](uint32_t p) {
				Page &s = pages[p];
				if (!on_cpu)
				{
					note_host(p);
					note_cache(p);
					s.host_write_pending |= r.block_mask;
					s.cached_read |= r.block_mask;
				}
				collect_dead(page_textures[p]);
				page_textures[p].push_back({ id, r.block_mask, r.write_mask, clut_instance });
			});
		}
		if (csa_mask != 0)
		{
			collect_dead(palette_textures);
			palette_textures.push_back({ id, csa_mask, UINT32_MAX, clut_instance });
		}
	}

	bool find_texture(uint64_t hash) const { return live.count(hash) != 0; }

	// invalidate_texture_cache (gs/page_tracker.cpp:911-941).
	void invalidate_texture_cache(uint32_t clut_instance)
	{
		bool any = false;
		for (uint16_t p : invalidate_pages)
		{
			Page &s = pages[p];
			if (!page_textures[p].empty())
				any = invalidate(page_textures[p], s.inv_block, s.inv_write, UINT32_MAX) || any;
			s.inv_block = 0;
			s.inv_write = 0;
		}
		invalidate_pages.clear();
		if (csa_written)
		{
			any = invalidate(palette_textures, csa_written, UINT32_MAX, clut_instance) || any;
			csa_written = 0;
		}
		if (any)
			client.tracker_texture_state_dirty_with_flush();
	}

	void invalidate_fb_write_short_term_references()
	{
		for (uint16_t p : fb_pages)
			if (!page_short_textures[p].empty())
				invalidate(page_short_textures[p], 0xffffffffu, pages[p].fb_write, UINT32_MAX);
	}

	// ---- flushes --------------------------------------------------------
	void flush_render_pass(uint32_t reason)
	{
		clear_cache_pages();
		clear_copy_pages();
		clear_fb_pages();
		invalidate_texture_cache(UINT32_MAX);
		client.tracker_flush(TRACKER_FLUSH_FB_ALL, reason);
	}

	// An explicit submission: pending host-visible state is settled
	// (mark_submission_timeline, gs/page_tracker.cpp:943-968).
	void mark_submission(uint32_t reason)
	{
		flush_render_pass(reason);
		for (uint16_t p : host_pages)
		{
			Page &s = pages[p];
			s.host_read_pending = 0;
			s.host_write_pending = 0;
		}
		host_pages.clear();
		client.tracker_flush(TRACKER_FLUSH_WRITE_BACK, reason);
	}

	void clear_cache_pages()
	{
		for (uint16_t p : cache_pages)
			pages[p].cached_read = 0;
		cache_pages.clear();
		client.tracker_forget_memoization();
	}

	void clear_copy_pages()
	{
		for (uint16_t p : copy_pages)
		{
			pages[p].copy_read = 0;
			pages[p].copy_write = 0;
		}
		copy_pages.clear();
	}

	void mark_memory_pressure() { pressure = true; }
	bool memory_pressure() const { return pressure; }

	void flush_if_memory_pressure()
	{
		if (pressure)
		{
			pressure = false;
			flush_render_pass(PGS_FLUSH_PRESSURE);
		}
	}

	Status texture_status(uint32_t id) const { return textures[id].status; }

private:
	struct Page
	{
		uint32_t fb_write, fb_read, pending_fb;
		uint32_t cached_read, copy_write, copy_read;
		uint32_t inv_block, inv_write;
		uint32_t host_read_pending, host_write_pending;
		bool may_super_sample;
	};
	struct Masked
	{
		uint32_t id, block_mask, write_mask, clut_instance;
	};
	struct Texture
	{
		uint64_t hash;
		Status status;
	};
	struct Blocks
	{
		uint32_t cached_read, copy_write, copy_read;
	};

	TrackerClient &client;
	Page pages[TRACKER_PAGES];
	std::vector<Masked> page_textures[TRACKER_PAGES], page_short_textures[TRACKER_PAGES];
	std::vector<Masked> palette_textures;
	std::vector<Texture> textures;
	std::unordered_map<uint64_t, uint32_t> live;
	std::vector<uint16_t> fb_pages, cache_pages, copy_pages, host_pages, short_pages, invalidate_pages;
	uint32_t csa_written = 0;
	uint32_t fb_lo = UINT32_MAX, fb_hi = 0, fb_mask = 0;
	bool pressure = false;

	template <typename F>
	static void for_pages(const PageRect &r, F &&f)
	{
		for (uint32_t y = 0; y < r.page_height; y++)
			for (uint32_t x = 0; x < r.page_width; x++)
				f((r.base_page + y * r.page_stride + x) & (TRACKER_PAGES - 1));
	}

	Blocks blocks(const PageRect &r) const
	{
		Blocks b = {};
		for_pages(r, [&](uint32_t p) {
			b.cached_read |= pages[p].cached_read;
			b.copy_write |= pages[p].copy_write;
			b.copy_read |= pages[p].copy_read;
		});
		return b;
	}

	void note_fb(uint32_t p)
	{
		if (pages[p].fb_read == 0 && pages[p].fb_write == 0)
			fb_pages.push_back(uint16_t(p));
	}
	void note_cache(uint32_t p)
	{
		if (pages[p].cached_read == 0)
			cache_pages.push_back(uint16_t(p));
	}
	void note_copy(uint32_t p)
	{
		if (pages[p].copy_read == 0 && pages[p].copy_write == 0)
			copy_pages.push_back(uint16_t(p));
	}
	void note_host(uint32_t p)
	{
		if (pages[p].host_write_pending == 0 && pages[p].host_read_pending == 0)
			host_pages.push_back(uint16_t(p));
	}
	void note_invalidate(uint32_t p)
	{
		if (pages[p].inv_block == 0)
			invalidate_pages.push_back(uint16_t(p));
	}

	uint32_t new_texture(uint64_t hash)
	{
		textures.push_back({ hash, LIVE });
		return uint32_t(textures.size() - 1);
	}

	void collect_dead(std::vector<Masked> &list)
	{
		size_t n = 0;
		for (size_t i = 0; i < list.size(); i++)
			if (textures[list[i].id].status != DEAD)
				list[n++] = list[i];
		list.resize(n);
	}

	// invalidate_cached_textures (gs/page_tracker.cpp:862-909).  A CLUT-only
	// invalidation leaves a texture floating: it may still be used by the
	// pass with the same palette instance.
	bool invalidate(std::vector<Masked> &list, uint32_t block_mask, uint32_t write_mask, uint32_t clut_instance)
	{
		bool did = false;
		const bool clut = clut_instance != UINT32_MAX;
		size_t n = 0;
		for (size_t i = 0; i < list.size(); i++)
		{
			Masked &m = list[i];
			Texture &t = textures[m.id];
			const bool can = t.status == LIVE || (t.status == FLOATING && !clut);
			if (can && (m.block_mask & block_mask) && (m.write_mask & write_mask) &&
			    (!clut || m.clut_instance != clut_instance))
			{
				if (t.status == LIVE)
				{
					auto it = live.find(t.hash);
					if (it != live.end() && it->second == m.id)
						live.erase(it);
				}
				client.tracker_invalidate_texture(t.hash, clut);
				t.status = clut ? FLOATING : DEAD;
				did = true;
			}
			if (t.status != DEAD)
				list[n++] = m;
		}
		list.resize(n);
		return did;
	}

	void clear_fb_pages()
	{
		for (uint16_t p : fb_pages)
		{
			pages[p].fb_read = 0;
			pages[p].fb_write = 0;
			pages[p].pending_fb = 0;
		}
		fb_pages.clear();
		fb_lo = UINT32_MAX;
		fb_hi = 0;
		fb_mask = 0;
		for (uint16_t p : short_pages)
			page_short_textures[p].clear();
		short_pages.clear();
		for (auto &m : palette_textures)
			if (textures[m.id].status == FLOATING)
				textures[m.id].status = DEAD;
	}

	void flush_copy()
	{
		client.tracker_flush(TRACKER_FLUSH_COPY_ALL, PGS_FLUSH_COPY_HAZARD);
		clear_copy_pages();
	}

	void flush_cached()
	{
		client.tracker_flush(TRACKER_FLUSH_CACHE_ALL, PGS_FLUSH_TEXTURE_HAZARD);
		clear_copy_pages();
		clear_cache_pages();
	}
};
} // namespace pgs
