// ref_frontend.cpp -- TEST INFRASTRUCTURE ONLY.
//
// Runs the reference's own CPU frontend -- GSInterface (gs/gs_interface.cpp),
// its PageTracker (gs/page_tracker.cpp) and gs/gs_util.cpp, compiled unmodified
// from the reference's sources -- over a recording GSRenderer, and exports what
// the frontend hands its renderer as an event log behind a C ABI.  The product
// frontend (parallel-gs_gb300/csrc/frontend.cpp) is checked against this log:
// render-pass boundaries and flush reasons, instances, coarse tile sizes,
// primitive records, state vectors, texture descriptors, copies and CLUT loads.
//
// The reference's GSRenderer (gs/gs_renderer.cpp) is Vulkan code and cannot
// run here; this file defines the GSRenderer members the frontend calls.  Where
// a renderer member feeds a decision back into the frontend it is restated
// from the reference, with the line it follows:
//   update_palette_cache / mark_clut_read / rewind_clut_instance / the CLUT part
//   of flush_cache_upload (gs/gs_renderer.cpp:3364-3419, 3662, 3817-3818, 3821-3824)
//     -- CLUT instance numbering and the texture-cache clobber on a rewind;
//   compute_effective_texture_rect (gs/gs_renderer.cpp:1235-1265)
//     -- texture page rectangles;
//   copy_vram / flush_rendering / flush_readback / flush_host_vram_copy /
//   flush_submit statistics and check_flush_stats (gs/gs_renderer.cpp:864-895,
//   1096-1104, 1526, 1555, 2829-2867, 3000, 3280-3281, 3413)
//     -- the pending-work limits that make the frontend end a render pass
//        early (FlushReason::PressureFlush).  The two memory-size limits
//        (allocated image memory against a fraction of the device's memory
//        budget, and render-pass scratch memory) depend on the Vulkan device
//        and allocator and are not modelled: only the host payload of
//        transfers counts as scratch here.
// Everything else the renderer does (GPU work, images, read-back) is recorded
// or ignored.  Timelines complete at once: query_timeline returns the last
// submitted value.
#include "gs_interface.hpp"
#include "gs_util.hpp"

#include <cstring>
#include <memory>
#include <unordered_map>
#include <vector>

namespace ParallelGS
{
static constexpr uint32_t PGS_REF_MaxPendingCopies = 16 * 1024;
static constexpr uint32_t PGS_REF_MaxPendingCopyThreads = 4 * 1024 * 1024;
static constexpr uint32_t PGS_REF_MaxPendingCopiesWithoutFlush = 1023;
static constexpr uint32_t PGS_REF_MinimumPrimitivesForFlush = 4096;
static constexpr uint32_t PGS_REF_MinimumRenderPassForFlush = 1024;
static constexpr uint32_t PGS_REF_MaxPendingPaletteUploads = 4096;
static constexpr uint64_t PGS_REF_MaximumAllocatedScratchMemory = 100ull * 1000 * 1000;

enum EventType : uint32_t
{
	EV_PASS = 1, EV_TEXTURE = 2, EV_COPY = 3, EV_PALETTE = 4, EV_FLUSH_CACHE = 5, EV_FLUSH_TRANSFER = 6,
	EV_SUBMIT = 7, EV_COPY_BARRIER = 8, EV_HOST_SYNC = 9, EV_READBACK = 10, EV_REWIND_CLUT = 11,
	EV_SET_SUPER_SAMPLING = 12, EV_SHADOW_PAGE = 13
};

struct Recorder
{
	std::vector<uint8_t> log;
	std::vector<VertexPosition> pos;
	std::vector<VertexAttribute> attr;
	std::vector<PrimitiveAttribute> prim;
	std::vector<uint8_t> host_vram;
	std::unordered_map<const Vulkan::Image *, uint32_t> image_ids;
	uint32_t next_image_id = 0;

	template <typename T>
	void put(const T &v)
	{
		const uint8_t *p = reinterpret_cast<const uint8_t *>(&v);
		log.insert(log.end(), p, p + sizeof(T));
	}
	void put_bytes(const void *p, size_t n)
	{
		const uint8_t *b = static_cast<const uint8_t *>(p);
		log.insert(log.end(), b, b + n);
	}
	// Every event: type, payload size, payload.
	size_t begin(uint32_t type)
	{
		put(type);
		size_t at = log.size();
		put(uint32_t(0));
		return at;
	}
	void end(size_t at)
	{
		uint32_t n = uint32_t(log.size() - at - 4);
		memcpy(log.data() + at, &n, 4);
	}
	void event(uint32_t type, const uint32_t *words, uint32_t n)
	{
		size_t at = begin(type);
		put_bytes(words, n * 4u);
		end(at);
	}
};

static std::unordered_map<const GSRenderer *, std::unique_ptr<Recorder>> g_recorders;

static Recorder &rec(const GSRenderer *r)
{
	auto &slot = g_recorders[r];
	if (!slot)
		slot.reset(new Recorder());
	return *slot;
}

// The renderer constructed last on this thread: GSInterface keeps its
// renderer private, so the harness picks it up here after construction.
static thread_local const GSRenderer *g_last_renderer = nullptr;

GSRenderer::GSRenderer(PageTracker &tracker_)
	: tracker(tracker_)
{
	g_last_renderer = this;
}

GSRenderer::~GSRenderer()
{
	g_recorders.erase(this);
}

bool GSRenderer::init(Vulkan::Device *, const GSOptions &options)
{
	vram_size = options.vram_size;
	vram_copy_write_pages.resize(vram_size / PageSize / 32);
	rec(this).host_vram.assign(vram_size, 0);
	return true;
}

void GSRenderer::reserve_primitive_buffers(uint32_t num_primitives)
{
	auto &r = rec(this);
	if (r.prim.size() < num_primitives)
	{
		r.pos.resize(3 * size_t(num_primitives));
		r.attr.resize(3 * size_t(num_primitives));
		r.prim.resize(num_primitives);
	}
	buffers.pos = r.pos.data();
	buffers.attr = r.attr.data();
	buffers.prim = r.prim.data();
}

VertexPosition *GSRenderer::get_reserved_vertex_positions() const { return buffers.pos; }
VertexAttribute *GSRenderer::get_reserved_vertex_attributes() const { return buffers.attr; }
PrimitiveAttribute *GSRenderer::get_reserved_primitive_attributes() const { return buffers.prim; }

void GSRenderer::check_flush_stats()
{
	if (stats.num_primitives >= PGS_REF_MinimumPrimitivesForFlush ||
	    stats.num_render_passes >= PGS_REF_MinimumRenderPassForFlush ||
	    stats.allocated_scratch_memory >= PGS_REF_MaximumAllocatedScratchMemory ||
	    stats.num_copies >= PGS_REF_MaxPendingCopies ||
	    stats.num_palette_updates >= PGS_REF_MaxPendingPaletteUploads)
	{
		tracker.mark_memory_pressure();
	}
	else if (pending_copies.size() >= PGS_REF_MaxPendingCopiesWithoutFlush ||
	         stats.num_copy_threads >= PGS_REF_MaxPendingCopyThreads)
	{
		flush_transfer();
	}
}

void GSRenderer::flush_host_vram_copy(const uint32_t *, uint32_t num_indices)
{
	uint32_t w[1] = { num_indices };
	rec(this).event(EV_HOST_SYNC, w, 1);
	stats.num_copies++;
	check_flush_stats();
}

uint32_t GSRenderer::update_palette_cache(const PaletteUploadDescriptor &desc)
{
	if (!last_clut_update_is_read && !palette_uploads.empty() &&
	    desc.fully_replaces_clut_upload(palette_uploads.back()))
	{
		uint32_t old_incoming = palette_uploads.back().incoming_clut_instance;
		palette_uploads.back() = desc;
		palette_uploads.back().incoming_clut_instance = old_incoming;
	}
	else
	{
		next_clut_instance = (next_clut_instance + 1) % CLUTInstances;
		palette_uploads.push_back(desc);
		stats.num_palette_updates++;
	}
	last_clut_update_is_read = false;

	auto &r = rec(this);
	size_t at = r.begin(EV_PALETTE);
	r.put(desc.tex0.bits);
	r.put(desc.texclut.bits);
	r.put(desc.csm2_x_bias);
	r.put(desc.csm2_x_scale);
	r.put(desc.csm1_reference_base);
	r.put(desc.csm1_mask);
	r.put(desc.incoming_clut_instance);
	r.put(next_clut_instance);
	r.end(at);

	check_flush_stats();
	return next_clut_instance;
}

bool PaletteUploadDescriptor::fully_replaces_clut_upload(const PaletteUploadDescriptor &old) const
{
	bool is_8bit = tex0.desc.PSM == PSMT8 || tex0.desc.PSM == PSMT8H;
	bool old_is_8bit = old.tex0.desc.PSM == PSMT8 || old.tex0.desc.PSM == PSMT8H;
	return old.tex0.desc.CPSM == tex0.desc.CPSM && old.tex0.desc.CSA == tex0.desc.CSA && is_8bit == old_is_8bit;
}

void GSRenderer::mark_clut_read(uint32_t clut_instance)
{
	if (clut_instance == next_clut_instance)
		last_clut_update_is_read = true;
}

void GSRenderer::rewind_clut_instance(uint32_t index)
{
	assert(palette_uploads.empty());
	if (index != next_clut_instance)
	{
		PageRectCLUT clut = {};
		clut.csa_mask = UINT32_MAX;
		tracker.register_cached_clut_clobber(clut);
		tracker.invalidate_texture_cache(index);
		uint32_t w[2] = { index, next_clut_instance };
		rec(this).event(EV_REWIND_CLUT, w, 2);
	}
	base_clut_instance = index;
	next_clut_instance = index;
}

TexRect GSRenderer::compute_effective_texture_rect(const TextureDescriptor &desc)
{
	uint32_t width_log2 = std::min<uint32_t>(desc.tex0.desc.TW, TEX0Bits::MAX_SIZE_LOG2);
	uint32_t height_log2 = std::min<uint32_t>(desc.tex0.desc.TH, TEX0Bits::MAX_SIZE_LOG2);
	uint32_t w = 1u << width_log2, h = 1u << height_log2;
	uint32_t max_levels = std::min<uint32_t>(TEX0Bits::MAX_LEVELS, std::min<uint32_t>(width_log2, height_log2) + 1);
	uint32_t levels = std::min<uint32_t>(uint32_t(desc.tex1.desc.MXL) + 1, max_levels);
	auto u = compute_effective_texture_extent(w, uint32_t(desc.clamp.desc.WMS), uint32_t(desc.clamp.desc.MINU),
	                                          uint32_t(desc.clamp.desc.MAXU), levels);
	auto v = compute_effective_texture_extent(h, uint32_t(desc.clamp.desc.WMT), uint32_t(desc.clamp.desc.MINV),
	                                          uint32_t(desc.clamp.desc.MAXV), levels);
	return { u.base, v.base, u.extent, v.extent, levels };
}

Vulkan::ImageHandle GSRenderer::create_cached_texture(const TextureDescriptor &desc)
{
	auto &r = rec(this);
	Vulkan::ImageHandle img(new Vulkan::Image(desc.rect.width, desc.rect.height, desc.rect.levels));
	uint32_t id = r.next_image_id++;
	r.image_ids[img.get()] = id;
	texture_uploads.push_back({});
	texture_uploads.back().image = img;
	texture_uploads.back().desc = desc;

	size_t at = r.begin(EV_TEXTURE);
	r.put(id);
	r.put(desc.tex0.bits);
	r.put(desc.tex1.bits);
	r.put(desc.miptbp1_3.bits);
	r.put(desc.miptbp4_6.bits);
	r.put(desc.texa.bits);
	r.put(desc.clamp.bits);
	r.put(desc.palette_bank);
	r.put(desc.samples);
	r.put(desc.rect.x);
	r.put(desc.rect.y);
	r.put(desc.rect.width);
	r.put(desc.rect.height);
	r.put(desc.rect.levels);
	r.end(at);
	return img;
}

void GSRenderer::promote_cached_texture_upload_cpu(const PageRect &) {}

void GSRenderer::commit_cached_texture(uint32_t, bool)
{
	check_flush_stats();
}

Vulkan::ImageHandle GSRenderer::copy_cached_texture(const Vulkan::Image &img, const VkRect2D &)
{
	auto &r = rec(this);
	Vulkan::ImageHandle copy(new Vulkan::Image(img.width, img.height, img.info.levels));
	auto it = r.image_ids.find(&img);
	r.image_ids[copy.get()] = it != r.image_ids.end() ? it->second : UINT32_MAX;
	return copy;
}

void GSRenderer::recycle_image_handle(Vulkan::ImageHandle) {}

void GSRenderer::flush_cache_upload()
{
	tracker.clear_cache_pages();
	// flush_palette_upload: the ring's committed base moves to the newest load.
	if (!palette_uploads.empty())
	{
		base_clut_instance = next_clut_instance;
		palette_uploads.clear();
	}
	texture_uploads.clear();
	rec(this).event(EV_FLUSH_CACHE, nullptr, 0);
}

void GSRenderer::copy_vram(const CopyDescriptor &desc, const PageRect &)
{
	stats.num_copy_threads += desc.trxreg.desc.RRW * desc.trxreg.desc.RRH;
	if (stats.num_copy_threads > PGS_REF_MaxPendingCopyThreads)
		flush_transfer();
	if (desc.trxdir.desc.XDIR == HOST_TO_LOCAL)
		stats.allocated_scratch_memory += desc.host_data_size;
	pending_copies.push_back({ desc, {} });

	auto &r = rec(this);
	size_t at = r.begin(EV_COPY);
	r.put(desc.bitbltbuf.bits);
	r.put(desc.trxpos.bits);
	r.put(desc.trxreg.bits);
	r.put(desc.trxdir.bits);
	r.put(uint64_t(desc.host_data_size));
	r.put(uint64_t(desc.host_data_size_offset));
	r.put(uint64_t(desc.host_data_size_required));
	r.put(uint32_t(desc.needs_shadow_vram));
	if (desc.trxdir.desc.XDIR == HOST_TO_LOCAL && desc.host_data)
		r.put_bytes(desc.host_data, desc.host_data_size);
	r.end(at);

	stats.num_copies++;
	check_flush_stats();
}

void GSRenderer::flush_transfer()
{
	pending_copies.clear();
	rec(this).event(EV_FLUSH_TRANSFER, nullptr, 0);
}

void GSRenderer::transfer_overlap_barrier()
{
	stats.num_copy_barriers++;
	rec(this).event(EV_COPY_BARRIER, nullptr, 0);
}

void GSRenderer::mark_shadow_page_sync(uint32_t page_index)
{
	rec(this).event(EV_SHADOW_PAGE, &page_index, 1);
}

void GSRenderer::flush_rendering(const RenderPass &rp)
{
	if (rp.num_primitives == 0)
		return;
	auto &r = rec(this);
	size_t at = r.begin(EV_PASS);
	r.put(uint32_t(rp.flush_reason));
	r.put(rp.num_primitives);
	r.put(rp.num_states);
	r.put(rp.num_textures);
	r.put(rp.num_instances);
	r.put(rp.coarse_tile_size_log2);
	r.put(uint32_t(rp.has_aa1));
	r.put(uint32_t(rp.has_scanmsk));
	r.put(uint32_t(rp.allow_blend_demote));
	r.put(uint32_t(rp.feedback_mode));
	r.put(rp.feedback_texture_psm);
	r.put(rp.feedback_texture_cpsm);
	for (uint32_t i = 0; i < rp.num_instances; i++)
	{
		auto &inst = rp.instances[i];
		r.put(inst.fb.frame.bits);
		r.put(inst.fb.z.bits);
		r.put(inst.base_x);
		r.put(inst.base_y);
		r.put(inst.coarse_tiles_width);
		r.put(inst.coarse_tiles_height);
		r.put(inst.opaque_fbmask);
		r.put(inst.sampling_rate_x_log2);
		r.put(inst.sampling_rate_y_log2);
		r.put(uint32_t(inst.z_sensitive));
		r.put(uint32_t(inst.z_write));
		r.put(uint32_t(inst.channel_shuffle));
	}
	r.put_bytes(buffers.pos, 3 * sizeof(VertexPosition) * rp.num_primitives);
	r.put_bytes(buffers.attr, 3 * sizeof(VertexAttribute) * rp.num_primitives);
	r.put_bytes(buffers.prim, sizeof(PrimitiveAttribute) * rp.num_primitives);
	r.put_bytes(rp.states, sizeof(StateVector) * rp.num_states);
	for (uint32_t i = 0; i < rp.num_textures; i++)
	{
		const auto &t = rp.textures[i];
		uint32_t id = UINT32_MAX;
		if (t.view && t.view->image)
		{
			auto it = r.image_ids.find(t.view->image);
			if (it != r.image_ids.end())
				id = it->second;
		}
		r.put(id);
		r.put(t.info);
	}
	r.end(at);

	// One shading dispatch per instance (gs/gs_renderer.cpp:3000); the
	// hazard-split dispatches of aliased instances are not counted.
	stats.num_render_passes += rp.num_instances;
	stats.num_primitives += rp.num_primitives;
	check_flush_stats();
}

void GSRenderer::flush_readback(const uint32_t *, uint32_t num_indices)
{
	uint32_t w[1] = { num_indices };
	rec(this).event(EV_READBACK, w, 1);
	stats.num_copies++;
	check_flush_stats();
}

void GSRenderer::flush_submit(uint64_t timeline)
{
	stats = {};
	last_submitted_timeline = timeline;
	uint32_t w[2] = { uint32_t(timeline), uint32_t(timeline >> 32) };
	rec(this).event(EV_SUBMIT, w, 2);
}

void GSRenderer::wait_timeline(uint64_t) {}
uint64_t GSRenderer::query_timeline() { return last_submitted_timeline; }
void *GSRenderer::begin_host_vram_access() { return rec(this).host_vram.data(); }
void GSRenderer::end_host_write_vram_access() {}

ScanoutResult GSRenderer::vsync(const PrivRegisterState &, const VSyncInfo &, uint32_t, uint32_t,
                                const Vulkan::Image *, const Vulkan::Image *)
{
	return {};
}

bool GSRenderer::vsync_can_skip(const PrivRegisterState &, const VSyncInfo &) const { return false; }
FlushStats GSRenderer::consume_flush_stats() { return {}; }
double GSRenderer::get_accumulated_timestamps(TimestampType) const { return 0.0; }
void GSRenderer::set_enable_timestamps(bool) {}

void GSRenderer::invalidate_super_sampling_state(uint32_t x, uint32_t y)
{
	uint32_t w[2] = { x, y };
	rec(this).event(EV_SET_SUPER_SAMPLING, w, 2);
}

SuperSampling GSRenderer::get_max_supported_super_sampling() const { return SuperSampling::X16; }
void GSRenderer::set_field_aware_super_sampling(bool enable) { field_aware_super_sampling = enable; }
}

using namespace ParallelGS;

struct pgs_ref_frontend
{
	GSInterface gs;
	const GSRenderer *renderer = nullptr;
};

extern "C" {
void *pgs_ref_frontend_create(uint32_t super_sampling, uint32_t ordered, uint32_t super_sampled_textures)
{
	auto *f = new pgs_ref_frontend();
	f->renderer = ParallelGS::g_last_renderer;
	GSOptions opts = {};
	opts.super_sampling = SuperSampling(super_sampling ? super_sampling : 1);
	opts.ordered_super_sampling = ordered != 0;
	opts.super_sampled_textures = super_sampled_textures != 0;
	if (!f->gs.init(nullptr, opts))
	{
		delete f;
		return nullptr;
	}
	return f;
}

void pgs_ref_frontend_destroy(void *f)
{
	delete static_cast<pgs_ref_frontend *>(f);
}

void pgs_ref_frontend_gif_transfer(void *f, uint32_t path, const void *data, size_t size)
{
	static_cast<pgs_ref_frontend *>(f)->gs.gif_transfer(path, data, size);
}

void pgs_ref_frontend_write_register(void *f, uint32_t addr, uint64_t value)
{
	static_cast<pgs_ref_frontend *>(f)->gs.write_register(RegisterAddr(addr), value);
}

void pgs_ref_frontend_flush(void *f)
{
	static_cast<pgs_ref_frontend *>(f)->gs.flush();
}

void pgs_ref_frontend_set_hacks(void *f, uint32_t disable_mipmaps, uint32_t allow_blend_demote)
{
	Hacks h = {};
	h.disable_mipmaps = disable_mipmaps != 0;
	h.allow_blend_demote = allow_blend_demote != 0;
	static_cast<pgs_ref_frontend *>(f)->gs.set_hacks(h);
}

void pgs_ref_frontend_set_super_sampling_rate(void *f, uint32_t super_sampling, uint32_t ordered,
                                              uint32_t super_sampled_textures)
{
	static_cast<pgs_ref_frontend *>(f)->gs.set_super_sampling_rate(SuperSampling(super_sampling), ordered != 0,
	                                                               super_sampled_textures != 0);
}

// The event log recorded so far (type u32, payload bytes u32, payload).
size_t pgs_ref_frontend_log_size(void *f)
{
	return ParallelGS::rec(static_cast<pgs_ref_frontend *>(f)->renderer).log.size();
}

const void *pgs_ref_frontend_log_data(void *f)
{
	return ParallelGS::rec(static_cast<pgs_ref_frontend *>(f)->renderer).log.data();
}

void pgs_ref_frontend_log_clear(void *f)
{
	ParallelGS::rec(static_cast<pgs_ref_frontend *>(f)->renderer).log.clear();
}
}
