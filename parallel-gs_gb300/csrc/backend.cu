// backend.cu -- CUDA implementation of pgs_backend_ops (the GSRenderer
// replacement, gs/gs_renderer.hpp:244-323) on one GB300.
//
// Memory in HBM:
//   VRAM    (2 + 2^max_samples_log2) x 4 MiB planes when super-sampling is
//           possible (plane 0 = GS local memory, plane 1 = super-sample
//           reference flags, planes 2.. = samples), else one plane
//           (gs/gs_renderer.cpp:360-427 minus the shadow half).
//   CLUT    1024 instances x 1 KiB ring (gs/gs_renderer.hpp:158-160).
//   arena   device mirror of a pinned host arena holding primitive records,
//           state vectors, texture descriptors and transfer payloads; every op
//           copies its own slice host->device once.  Recorded frames replay
//           straight from the device arena.
//   scratch per-pass setup records, per-tile primitive bitmasks and flags.
//
// Everything runs in order on one CUDA stream.  Kernels never wait on other
// kernels or on the host, so no launch can hang.
#include "kernels.cuh"

#include <algorithm>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <new>
#include <vector>

using namespace pgs;

namespace
{
#define CUDA_TRY(expr)                                                                   \
	do                                                                                   \
	{                                                                                    \
		cudaError_t e_ = (expr);                                                         \
		if (e_ != cudaSuccess)                                                           \
		{                                                                                \
			fprintf(stderr, "pgs: %s failed: %s\n", #expr, cudaGetErrorString(e_));     \
			return PGS_ERROR_CUDA;                                                       \
		}                                                                                \
	} while (0)

const uint8_t RCP_TABLE[256] = {
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

inline size_t align_up(size_t v, size_t a) { return (v + a - 1) & ~(a - 1); }

enum OpType : uint32_t { OP_COPY = 0, OP_CLUT = 1, OP_PASS = 2, OP_SNAPSHOT = 3 };

struct PassOp
{
	size_t pos_off, attr_off, prim_off, states_off, textures_off, images_off;
	uint32_t num_texels, max_texels, max_levels;
	uint32_t num_prims, num_states, num_textures;
	uint32_t tile_size_log2, has_aa1, has_scanmsk, has_mipmap, has_ss_textures;
	uint32_t rp_is_blur_mask;
	uint32_t field_aware;   // pgs_render_pass.field_aware
	uint32_t blend_demote;  // primitives per coarse tile that demote a blended tile, 0 = off
	uint32_t num_instances;
	pgs_rp_instance instances[PGS_MAX_RENDER_PASS_INSTANCES];
	// Textures [snap_limit[k - 1], snap_limit[k]) decode from snapshot slot k.
	uint32_t num_snaps;
	uint32_t snap_limit[PGS_MAX_VRAM_SNAPSHOTS];
	// Host copy of the primitive records while the pass is submitted
	// (null for recorded passes, which keep theirs in the host arena).
	const pgs_primitive_attribute *host_prims;
};

struct Op
{
	OpType type;
	CopyParams copy;
	size_t copy_host_off;
	ClutParams clut;
	PassOp pass;
	uint32_t snap_slot;
};

struct Dispatch
{
	DevInstance inst;
	uint32_t num_tiles;
};

// Phase LUT of super-sampled texture filtering (GSRenderer::init_phase_lut,
// gs/gs_renderer.cpp:93-315): for each of 64 x 64 sub-texel phases, the four
// nearest (sample, texel offset) points of the sampling grid -- the first one
// always in the centre texel -- with tent weights over the falloff distance in
// unorm8 summing to 255; for 32 x 32 phases, the nearest sample (nearest
// filtering).  Ties in the distance order keep generation order.
static void build_phase_lut(uint32_t rx, uint32_t ry, uint32_t *lut)
{
	std::fill(lut, lut + PHASE_LUT_WORDS, 0u);
	if (!rx && !ry)
		return;
	constexpr int G = 64;
	const int n = 1 << (rx + ry);
	struct Pt { int x, y; };
	auto points = [&](Pt *out, bool nearest) {
		for (int i = 0; i < n; i++)
		{
			int x, y;
			if (int(ry) - int(rx) == 2)
			{
				static const int sparse[4] = { 0, 2, 3, 1 };
				x = (i / 8) * 4 + sparse[i % 4];
				y = i % 8;
			}
			else
			{
				y = (i & 1) + ((i >> 2) & 1) * 2;
				x = ((i >> 1) & 1) + ((i >> 3) & 1) * 2;
				if (int(ry) - int(rx) == 1)
					x = x * 2 + i % 2;
			}
			const int scale = G >> ry;
			x *= scale;
			y *= scale;
			if (nearest)
			{
				x += (scale - 1) >> 1;
				y += (scale - 1) >> 1;
			}
			out[i] = { x, y };
		}
	};
	struct Cand { int sample, ox, oy, dx, dy, maxd; };
	auto candidates = [&](int x, int y, const Pt *pts, int support, std::vector<Cand> &out) {
		out.clear();
		for (int i = 0; i < n; i++)
			for (int ty = -support; ty <= support; ty++)
				for (int tx = -support; tx <= support; tx++)
				{
					const int dx = std::abs(pts[i].x + G * tx - x), dy = std::abs(pts[i].y + G * ty - y);
					out.push_back({ i, tx, ty, dx, dy, std::max(dx, dy) });
				}
		std::stable_sort(out.begin(), out.end(), [](const Cand &a, const Cand &b) {
			return a.maxd == b.maxd ? a.dy < b.dy : a.maxd < b.maxd;
		});
	};
	Pt pts[16], pts_nearest[16];
	points(pts, false);
	points(pts_nearest, true);
	std::vector<Cand> c;
	int falloff = INT32_MAX;
	for (int y = 0; y < G; y++)
		for (int x = 0; x < G; x++)
		{
			candidates(x, y, pts, 1, c);
			falloff = std::min(falloff, c[4].maxd);
		}
	for (int y = 0; y < G; y++)
		for (int x = 0; x < G; x++)
		{
			candidates(x, y, pts, 1, c);
			if (c[0].ox != 0 || c[0].oy != 0)
			{
				for (size_t i = 1; i < c.size(); i++)
				{
					if (c[i].ox == 0 && c[i].oy == 0)
					{
						if (i < 4)
							std::swap(c[0], c[i]);
						else
						{
							std::swap(c[3], c[i]);
							std::swap(c[0], c[3]);
						}
						break;
					}
				}
			}
			uint32_t ex = 0, ey = 0;
			float w[4], sum = 0.0f;
			for (int i = 0; i < 4; i++)
			{
				ex |= uint32_t(c[i].sample) << (4 * i);
				ex |= (uint32_t(c[i].ox) & 3u) << (4 * i + 16);
				ex |= (uint32_t(c[i].oy) & 3u) << (4 * i + 18);
				const float fx = float(c[i].dx) / float(falloff), fy = float(c[i].dy) / float(falloff);
				w[i] = std::max(0.0f, 1.0f - fx) * std::max(0.0f, 1.0f - fy);
				sum += w[i];
			}
			if (sum < 0.001f)
			{
				for (float &v : w)
					v = 1.0f;
				sum = 4.0f;
			}
			uint32_t total = 0;
			for (int i = 0; i < 3; i++)
			{
				const float scaled = w[i] * 255.0f / sum;
				uint32_t q = uint32_t(scaled + 0.5f);
				q = std::min<uint32_t>(q, 255u - total);
				total += q;
				ey |= q << (8 * i);
			}
			ey |= (255u - total) << 24;
			lut[(y * G + x) * 2] = ex;
			lut[(y * G + x) * 2 + 1] = ey;
		}
	for (int y = 0; y < G / 2; y++)
		for (int x = 0; x < G / 2; x++)
		{
			candidates(2 * x, 2 * y, pts_nearest, 0, c);
			lut[G * G * 2 + y * (G / 2) + x] = uint32_t(c[0].sample);
		}
}

struct CudaBackend
{
	int device = 0;
	cudaStream_t stream = nullptr;
	uint32_t max_planes = 1;
	uint32_t num_planes = 1;
	uint32_t rate_x = 0, rate_y = 0;

	uint8_t *d_vram = nullptr;
	uint16_t *d_clut = nullptr;
	float *d_rcp_float = nullptr;
	float *d_unorm_lut = nullptr;
	uint32_t *d_phase_lut = nullptr; // PHASE_LUT_WORDS, for the current sampling rate
	uint32_t *d_error = nullptr;
	unsigned long long *d_frags = nullptr;
	uint8_t *d_snapshot = nullptr;
	// VRAM snapshots of the open render pass (snapshot_vram): every plane,
	// allocated on first use; snapshots_taken counts the pass's slots in use.
	uint8_t *d_tex_snap[PGS_MAX_VRAM_SNAPSHOTS] = {};
	uint32_t snapshots_taken = 0;
	uint32_t last_clut = 0;

	// Arena.
	uint8_t *h_arena = nullptr, *d_arena = nullptr;
	size_t arena_cap = 0, arena_used = 0;

	// Reserved primitive buffers (pinned).  Two to start with, so that the
	// frontend fills one while the other is copied; when every buffer still
	// waits for its copy (the copies queue behind the passes before them), one
	// more is added, up to MAX_STAGES, so that a frame of many passes is
	// recorded ahead of the device instead of in step with it.
	static constexpr int MAX_STAGES = 6;
	uint8_t *h_stage[MAX_STAGES] = {};
	cudaEvent_t stage_done[MAX_STAGES] = {};
	int stage_index = 0, num_stages = 0;
	bool stage_pending[MAX_STAGES] = {};

	// Scratch.
	PrimSetup *d_setup = nullptr;
	TransformedAttr *d_tattr = nullptr;
	pgs_primitive_attribute *d_prims_work = nullptr;
	SsHeuristic *d_heuristic = nullptr;
	uint8_t *d_heuristic_action = nullptr;
	uint32_t *d_masks = nullptr;
	size_t masks_cap = 0;
	uint32_t *d_flags = nullptr;
	size_t flags_cap = 0;
	uint32_t *d_texels = nullptr;
	size_t texels_cap = 0;
	uint32_t *d_circuit = nullptr;
	uint8_t *d_readback = nullptr;
	uint64_t readback_cap = 0;
	uint8_t *d_zcache = nullptr; // depth snapshot for aliased frame / depth buffers
	size_t zcache_cap = 0;
	// vsync: circuit read-outs, merged image, output and the last four
	// merged fields for the deinterlacer (slot order: newest first).
	struct DevImage
	{
		uint32_t *ptr = nullptr;
		size_t cap = 0;
	};
	DevImage vs_circuit[2], vs_merged, vs_out, vs_fields[4];
	bool vs_field_valid[4] = {};
	uint32_t vs_field_w = 0, vs_field_h = 0;
	size_t circuit_cap = 0;

	// Recording.
	bool recording = false;
	std::vector<Op> ops;
	std::vector<uint64_t> batch_blocks;
	std::vector<uint32_t> scratch_blocks;
	uint8_t *d_reset_vram = nullptr;
	uint16_t *d_reset_clut = nullptr;
	uint32_t reset_planes = 0;
	cudaGraphExec_t graph_exec = nullptr;
	uint32_t launches_per_replay = 0;
	uint32_t launch_counter = 0;
	cudaEvent_t shade_ev[2] = {};
	float last_shade_ms = 0.0f;
	bool shade_timing = false;
	bool shade_started = false;

	// Stage timestamps (GSRenderer timestamps, gs/gs_renderer.cpp:1205-1233):
	// while on, each stage issued outside stream capture is bracketed by an
	// event pair; the pairs are summed per stage when the totals are read.
	struct StageSpan
	{
		uint32_t type;
		cudaEvent_t ev[2];
	};
	bool stage_timing = false;
	std::vector<StageSpan> stage_spans;
	std::vector<cudaEvent_t> stage_events; // free events
	double stage_total[PGS_TIMESTAMP_COUNT] = {};

	bool stage_begin(uint32_t type, StageSpan &sp)
	{
		if (!stage_timing)
			return false;
		cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
		if (cudaStreamIsCapturing(stream, &cs) != cudaSuccess || cs != cudaStreamCaptureStatusNone)
			return false;
		while (stage_events.size() < 2)
		{
			cudaEvent_t e = nullptr;
			if (cudaEventCreate(&e) != cudaSuccess)
				return false;
			stage_events.push_back(e);
		}
		sp.type = type;
		sp.ev[0] = stage_events.back();
		stage_events.pop_back();
		sp.ev[1] = stage_events.back();
		stage_events.pop_back();
		cudaEventRecord(sp.ev[0], stream);
		return true;
	}

	void stage_end(const StageSpan &sp)
	{
		cudaEventRecord(sp.ev[1], stream);
		stage_spans.push_back(sp);
		if (stage_spans.size() >= 4096)
			stage_collect();
	}

	int stage_collect()
	{
		int r = PGS_OK;
		for (const auto &sp : stage_spans)
		{
			float ms = 0.0f;
			if (r == PGS_OK && cudaEventSynchronize(sp.ev[1]) == cudaSuccess &&
			    cudaEventElapsedTime(&ms, sp.ev[0], sp.ev[1]) == cudaSuccess)
				stage_total[sp.type] += double(ms) * 1e-3;
			else
				r = PGS_ERROR_CUDA;
			stage_events.push_back(sp.ev[0]);
			stage_events.push_back(sp.ev[1]);
		}
		stage_spans.clear();
		return r;
	}

	// Brackets the work issued in its scope as one span of `type`.
	struct StageScope
	{
		CudaBackend *b;
		StageSpan sp;
		bool on;
		StageScope(CudaBackend *b_, uint32_t type) : b(b_), on(b_->stage_begin(type, sp)) {}
		~StageScope() { if (on) b->stage_end(sp); }
	};

	int timestamps(int enable, double *totals)
	{
		if (enable >= 0)
			stage_timing = enable != 0;
		if (!totals)
			return PGS_OK;
		int r = stage_collect();
		memcpy(totals, stage_total, sizeof(stage_total));
		return r;
	}
	uint64_t h2d_bytes = 0, d2h_bytes = 0, total_launches = 0, render_passes = 0;

	// Asynchronous readbacks in flight.  A destination outside pinned memory
	// is staged through a pinned slot and copied out by wait_ticket.
	static constexpr int READBACK_SLOTS = 4;
	struct Readback
	{
		uint64_t ticket = 0;
		cudaEvent_t done = nullptr;
		uint8_t *staging = nullptr;
		void *dst = nullptr;
		uint64_t size = 0;
	} readbacks[READBACK_SLOTS];
	uint64_t next_ticket = 1;

	// ------------------------------------------------------------------
	int init(const pgs_cuda_backend_options *opt)
	{
		int count = 0;
		if (cudaGetDeviceCount(&count) != cudaSuccess || count == 0)
			return PGS_ERROR_NO_DEVICE;
		device = opt ? opt->device : 0;
		if (device < 0 || device >= count)
			return PGS_ERROR_INVALID_ARGUMENT;
		CUDA_TRY(cudaSetDevice(device));
		CUDA_TRY(cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking));
		uint32_t ms = opt ? std::min<uint32_t>(opt->max_samples_log2, 4) : 4;
		max_planes = ms ? 2u + (1u << ms) : 1u;
		CUDA_TRY(cudaMalloc(&d_vram, size_t(max_planes) * VRAM_SIZE));
		CUDA_TRY(cudaMemset(d_vram, 0, size_t(max_planes) * VRAM_SIZE));
		CUDA_TRY(cudaMalloc(&d_clut, size_t(PGS_CLUT_INSTANCES) * PGS_CLUT_SIZE_BYTES));
		CUDA_TRY(cudaMemset(d_clut, 0, size_t(PGS_CLUT_INSTANCES) * PGS_CLUT_SIZE_BYTES));
		CUDA_TRY(cudaMalloc(&d_snapshot, VRAM_SIZE));
		CUDA_TRY(cudaMalloc(&d_error, sizeof(uint32_t)));
		CUDA_TRY(cudaMemset(d_error, 0, sizeof(uint32_t)));
		CUDA_TRY(cudaMalloc(&d_frags, sizeof(unsigned long long)));
		CUDA_TRY(cudaMemset(d_frags, 0, sizeof(unsigned long long)));

		float lut[256];
		for (int i = 0; i < 256; i++)
			lut[i] = 1.0f / (1.0f + (float(i) + 0.5f) / 256.0f);
		CUDA_TRY(cudaMalloc(&d_rcp_float, sizeof(lut)));
		CUDA_TRY(cudaMemcpy(d_rcp_float, lut, sizeof(lut), cudaMemcpyHostToDevice));
		// unpackUnorm4x8 table: float(c) / 255 with IEEE division on the host.
		volatile float denom = 255.0f;
		for (int i = 0; i < 256; i++)
			lut[i] = float(i) / denom;
		CUDA_TRY(cudaMalloc(&d_unorm_lut, sizeof(lut)));
		CUDA_TRY(cudaMemcpy(d_unorm_lut, lut, sizeof(lut), cudaMemcpyHostToDevice));
		CUDA_TRY(cudaMalloc(&d_phase_lut, PHASE_LUT_WORDS * sizeof(uint32_t)));
		CUDA_TRY(cudaMemset(d_phase_lut, 0, PHASE_LUT_WORDS * sizeof(uint32_t)));
		CUDA_TRY(cudaMemcpyToSymbol(c_rcp_tab, RCP_TABLE, sizeof(RCP_TABLE)));

		const size_t n = PGS_MAX_PRIMITIVES_PER_FLUSH;
		CUDA_TRY(cudaMalloc(&d_setup, n * sizeof(PrimSetup)));
		CUDA_TRY(cudaMalloc(&d_tattr, n * sizeof(TransformedAttr)));
		CUDA_TRY(cudaMalloc(&d_prims_work, n * sizeof(pgs_primitive_attribute)));
		CUDA_TRY(cudaMalloc(&d_heuristic, sizeof(SsHeuristic)));
		CUDA_TRY(cudaMalloc(&d_heuristic_action, n));
		CUDA_TRY(cudaMemset(d_heuristic_action, 0, n));
		for (int i = 0; i < 2; i++)
		{
			int r = add_stage();
			if (r)
				return r;
			CUDA_TRY(cudaEventCreate(&shade_ev[i]));
		}
		for (auto &rb : readbacks)
			CUDA_TRY(cudaEventCreateWithFlags(&rb.done, cudaEventDisableTiming));
		return grow_arena(size_t(opt && opt->arena_mib ? opt->arena_mib : 256u) << 20);
	}

	int add_stage()
	{
		const int i = num_stages;
		if (cudaMallocHost(&h_stage[i], stage_bytes()) != cudaSuccess)
		{
			// Out of pinned memory is not fatal past the first two buffers:
			// the caller waits for one instead.
			(void)cudaGetLastError();
			h_stage[i] = nullptr;
			return PGS_ERROR_OUT_OF_MEMORY;
		}
		CUDA_TRY(cudaEventCreateWithFlags(&stage_done[i], cudaEventDisableTiming));
		stage_pending[i] = false;
		num_stages++;
		return PGS_OK;
	}

	static size_t stage_bytes()
	{
		const size_t n = PGS_MAX_PRIMITIVES_PER_FLUSH;
		return n * (3 * sizeof(pgs_vertex_position) + 3 * sizeof(pgs_vertex_attribute) + sizeof(pgs_primitive_attribute));
	}

	void destroy()
	{
		cudaSetDevice(device);
		if (stream)
			cudaStreamSynchronize(stream);
		if (graph_exec)
			cudaGraphExecDestroy(graph_exec);
		cudaFree(d_vram);
		cudaFree(d_clut);
		cudaFree(d_snapshot);
		for (auto &p : d_tex_snap)
		{
			cudaFree(p);
			p = nullptr;
		}
		cudaFree(d_error);
		cudaFree(d_frags);
		cudaFree(d_rcp_float);
		cudaFree(d_unorm_lut);
		cudaFree(d_setup);
		cudaFree(d_tattr);
		cudaFree(d_prims_work);
		cudaFree(d_heuristic);
		cudaFree(d_heuristic_action);
		cudaFree(d_masks);
		cudaFree(d_flags);
		cudaFree(d_texels);
		cudaFree(d_circuit);
		cudaFree(d_readback);
		cudaFree(d_zcache);
		cudaFree(d_phase_lut);
		for (DevImage *im : { &vs_circuit[0], &vs_circuit[1], &vs_merged, &vs_out, &vs_fields[0], &vs_fields[1],
		                      &vs_fields[2], &vs_fields[3] })
			cudaFree(im->ptr);
		cudaFree(d_arena);
		cudaFree(d_reset_vram);
		cudaFree(d_reset_clut);
		cudaFreeHost(h_arena);
		for (int i = 0; i < MAX_STAGES; i++)
		{
			if (h_stage[i]) cudaFreeHost(h_stage[i]);
			if (stage_done[i]) cudaEventDestroy(stage_done[i]);
		}
		for (int i = 0; i < 2; i++)
			if (shade_ev[i]) cudaEventDestroy(shade_ev[i]);
		for (auto &rb : readbacks)
		{
			if (rb.done) cudaEventDestroy(rb.done);
			cudaFreeHost(rb.staging);
		}
		for (const auto &sp : stage_spans)
		{
			cudaEventDestroy(sp.ev[0]);
			cudaEventDestroy(sp.ev[1]);
		}
		for (cudaEvent_t e : stage_events)
			cudaEventDestroy(e);
		if (stream)
			cudaStreamDestroy(stream);
	}

	int grow_arena(size_t need)
	{
		size_t cap = std::max<size_t>(arena_cap ? arena_cap * 2 : 0, need);
		uint8_t *h = nullptr, *d = nullptr;
		CUDA_TRY(cudaStreamSynchronize(stream));
		CUDA_TRY(cudaMallocHost(&h, cap));
		CUDA_TRY(cudaMalloc(&d, cap));
		if (arena_used)
		{
			memcpy(h, h_arena, arena_used);
			CUDA_TRY(cudaMemcpy(d, d_arena, arena_used, cudaMemcpyDeviceToDevice));
		}
		cudaFreeHost(h_arena);
		cudaFree(d_arena);
		h_arena = h;
		d_arena = d;
		arena_cap = cap;
		if (graph_exec)
		{
			cudaGraphExecDestroy(graph_exec);
			graph_exec = nullptr;
		}
		return PGS_OK;
	}

	// Appends `size` bytes to the arena and returns the offset.  Outside of
	// recording the arena restarts once the stream is idle.
	int arena_alloc(size_t size, size_t &off)
	{
		size = align_up(size, 256);
		if (arena_used + size > arena_cap)
		{
			if (!recording)
			{
				int r = flush_deferred();
				if (r)
					return r;
				CUDA_TRY(cudaStreamSynchronize(stream));
				arena_used = 0;
			}
			if (arena_used + size > arena_cap)
			{
				int r = grow_arena(arena_used + size);
				if (r)
					return r;
			}
		}
		off = arena_used;
		arena_used += size;
		return PGS_OK;
	}

	// Index of the staging buffer holding the render pass's records, or -1.
	int staging_buffer_of(const pgs_render_pass *rp) const
	{
		const size_t N = PGS_MAX_PRIMITIVES_PER_FLUSH;
		for (int i = 0; i < num_stages; i++)
		{
			const uint8_t *base = h_stage[i];
			if (reinterpret_cast<const uint8_t *>(rp->positions) == base &&
			    reinterpret_cast<const uint8_t *>(rp->attributes) == base + N * 3 * sizeof(pgs_vertex_position) &&
			    reinterpret_cast<const uint8_t *>(rp->prims) ==
			        base + N * 3 * (sizeof(pgs_vertex_position) + sizeof(pgs_vertex_attribute)))
				return i;
		}
		return -1;
	}

	int upload_arena(size_t off, size_t size)
	{
		if (size)
			CUDA_TRY(cudaMemcpyAsync(d_arena + off, h_arena + off, size, cudaMemcpyHostToDevice, stream));
		h2d_bytes += size;
		return PGS_OK;
	}

	// ------------------------------------------------------------------
	int reserve(uint32_t n, pgs_vertex_position **pos, pgs_vertex_attribute **attr, pgs_primitive_attribute **prim)
	{
		if (n > PGS_MAX_PRIMITIVES_PER_FLUSH)
			return PGS_ERROR_INVALID_ARGUMENT;
		// The next buffer whose copy has finished; else a new one; else wait
		// for the next in turn.
		int pick = -1;
		for (int k = 1; k <= num_stages && pick < 0; k++)
		{
			const int i = (stage_index + k) % num_stages;
			if (stage_pending[i])
			{
				const cudaError_t q = cudaEventQuery(stage_done[i]);
				if (q == cudaErrorNotReady)
				{
					// Not an error: keep it out of the launch checks' last error.
					if (cudaPeekAtLastError() == cudaErrorNotReady)
						(void)cudaGetLastError();
					continue;
				}
				CUDA_TRY(q);
				stage_pending[i] = false;
			}
			pick = i;
		}
		if (pick < 0 && num_stages < MAX_STAGES && add_stage() == PGS_OK)
			pick = num_stages - 1;
		if (pick < 0)
		{
			pick = (stage_index + 1) % num_stages;
			CUDA_TRY(cudaEventSynchronize(stage_done[pick]));
			stage_pending[pick] = false;
		}
		stage_index = pick;
		const size_t N = PGS_MAX_PRIMITIVES_PER_FLUSH;
		uint8_t *base = h_stage[stage_index];
		*pos = reinterpret_cast<pgs_vertex_position *>(base);
		*attr = reinterpret_cast<pgs_vertex_attribute *>(base + N * 3 * sizeof(pgs_vertex_position));
		*prim = reinterpret_cast<pgs_primitive_attribute *>(base + N * 3 * (sizeof(pgs_vertex_position) + sizeof(pgs_vertex_attribute)));
		return PGS_OK;
	}

	int flush_rendering(const pgs_render_pass *rp)
	{
		if (!rp)
			return PGS_OK;
		if (rp->num_primitives == 0)
		{
			// An empty pass only releases its snapshot slots.
			snapshots_taken = 0;
			return PGS_OK;
		}
		if (rp->num_primitives > PGS_MAX_PRIMITIVES_PER_FLUSH || rp->num_instances == 0 ||
		    rp->num_instances > PGS_MAX_RENDER_PASS_INSTANCES || rp->coarse_tile_size_log2 < 3 ||
		    rp->coarse_tile_size_log2 > 7)
			return PGS_ERROR_INVALID_ARGUMENT;

		Op op = {};
		op.type = OP_PASS;
		PassOp &p = op.pass;
		uint32_t n = rp->num_primitives;
		size_t pos_bytes = size_t(n) * 3 * sizeof(pgs_vertex_position);
		size_t attr_bytes = size_t(n) * 3 * sizeof(pgs_vertex_attribute);
		size_t prim_bytes = size_t(n) * sizeof(pgs_primitive_attribute);
		size_t st_bytes = size_t(std::max<uint32_t>(rp->num_states, 1)) * sizeof(pgs_state_vector);
		size_t tex_bytes = size_t(std::max<uint32_t>(rp->num_textures, 1)) * sizeof(pgs_texture_desc);
		size_t img_bytes = size_t(std::max<uint32_t>(rp->num_textures, 1)) * TEX_SLOTS * sizeof(TexImage);
		size_t base;
		size_t total = align_up(pos_bytes, 256) + align_up(attr_bytes, 256) + align_up(prim_bytes, 256) +
		               align_up(st_bytes, 256) + align_up(tex_bytes, 256) + align_up(img_bytes, 256);
		int r = arena_alloc(total, base);
		if (r)
			return r;
		p.pos_off = base;
		p.attr_off = p.pos_off + align_up(pos_bytes, 256);
		p.prim_off = p.attr_off + align_up(attr_bytes, 256);
		p.states_off = p.prim_off + align_up(prim_bytes, 256);
		p.textures_off = p.states_off + align_up(st_bytes, 256);
		// Records written by the frontend into a staging buffer go to the
		// device straight from there; a recorded frame keeps a host copy.
		int stage = recording ? -1 : staging_buffer_of(rp);
		if (stage >= 0)
		{
			CUDA_TRY(cudaMemcpyAsync(d_arena + p.pos_off, rp->positions, pos_bytes, cudaMemcpyHostToDevice, stream));
			CUDA_TRY(cudaMemcpyAsync(d_arena + p.attr_off, rp->attributes, attr_bytes, cudaMemcpyHostToDevice, stream));
			CUDA_TRY(cudaMemcpyAsync(d_arena + p.prim_off, rp->prims, prim_bytes, cudaMemcpyHostToDevice, stream));
			CUDA_TRY(cudaEventRecord(stage_done[stage], stream));
			stage_pending[stage] = true;
			h2d_bytes += pos_bytes + attr_bytes + prim_bytes;
			p.host_prims = rp->prims;
		}
		else
		{
			memcpy(h_arena + p.pos_off, rp->positions, pos_bytes);
			memcpy(h_arena + p.attr_off, rp->attributes, attr_bytes);
			memcpy(h_arena + p.prim_off, rp->prims, prim_bytes);
			p.host_prims = nullptr;
		}
		if (rp->num_states)
			memcpy(h_arena + p.states_off, rp->states, rp->num_states * sizeof(pgs_state_vector));
		if (rp->num_textures)
			memcpy(h_arena + p.textures_off, rp->textures, rp->num_textures * sizeof(pgs_texture_desc));
		p.images_off = p.textures_off + align_up(tex_bytes, 256);
		{
			// Decoded extent of each mip level covers every texel index the wrap
			// modes can produce at that level (region bounds scale with the level).
			TexImage *im = reinterpret_cast<TexImage *>(h_arena + p.images_off);
			memset(im, 0, img_bytes);
			uint64_t texels = 0;
			uint32_t max_texels = 0, max_levels = 1;
			for (uint32_t i = 0; i < rp->num_textures; i++)
			{
				const pgs_texture_desc &t = rp->textures[i];
				uint32_t levels = std::max<uint32_t>(t.levels, 1);
				if (levels > TEX_LEVELS || std::min(std::min(t.tw_log2, t.th_log2), 10u) + 1 < levels)
					return PGS_ERROR_INVALID_ARGUMENT;
				// Super-sampled textures: one level, a layer per sample the VRAM holds.
				if (t.samples > 1 && (levels != 1 || (t.samples & (t.samples - 1)) || t.samples > 16 ||
				                      2u + t.samples > num_planes))
					return PGS_ERROR_INVALID_ARGUMENT;
				const uint32_t slots = texture_slots(t);
				max_levels = std::max(max_levels, slots);
				for (uint32_t s = 0; s < slots; s++)
				{
					const uint32_t l = t.samples > 1 ? 0u : s;
					auto extent = [l](uint32_t size_log2, uint32_t mode, uint32_t lo, uint32_t hi) {
						uint32_t size = 1u << (std::min<uint32_t>(size_log2, 10) - l);
						lo >>= l;
						hi >>= l;
						if (mode == WRAP_REGION_CLAMP)
							return std::max(size, std::max(lo, hi) + 1u);
						if (mode == WRAP_REGION_REPEAT)
							return std::max(size, (((size - 1u) & lo) | hi) + 1u);
						return size;
					};
					TexImage &m = im[i * TEX_SLOTS + s];
					m.ext_u = extent(t.tw_log2, t.wms, t.minu, t.maxu);
					m.ext_v = extent(t.th_log2, t.wmt, t.minv, t.maxv);
					m.offset = uint32_t(texels);
					uint32_t n = m.ext_u * m.ext_v;
					texels += n;
					max_texels = std::max(max_texels, n);
				}
			}
			if (texels > (uint64_t(1) << 31))
				return PGS_ERROR_CAPACITY;
			p.num_texels = uint32_t(texels);
			p.max_texels = max_texels;
			p.max_levels = max_levels;
		}
		r = stage >= 0 ? upload_arena(p.states_off, total - (p.states_off - base)) : upload_arena(base, total);
		if (r)
			return r;

		p.num_prims = n;
		p.num_states = rp->num_states;
		p.num_textures = rp->num_textures;
		p.tile_size_log2 = rp->coarse_tile_size_log2;
		p.has_aa1 = rp->has_aa1;
		p.has_mipmap = rp->has_mipmap;
		p.has_ss_textures = rp->has_ss_textures;
		p.rp_is_blur_mask = blur_mask(rp);
		p.field_aware = rp->field_aware;
		p.blend_demote = blend_demote_budget(rp);
		p.has_scanmsk = rp->has_scanmsk;
		p.num_instances = rp->num_instances;
		memcpy(p.instances, rp->instances, sizeof(p.instances));
		p.num_snaps = std::min<uint32_t>(rp->num_snapshots, snapshots_taken);
		for (uint32_t k = 0; k < p.num_snaps; k++)
			p.snap_limit[k] = std::min(rp->snapshot_textures[k], rp->num_textures);
		snapshots_taken = 0;
		return submit(op);
	}

	// snapshot_vram: all planes into the pass's next slot, in stream order.
	int snapshot_vram()
	{
		if (snapshots_taken >= PGS_MAX_VRAM_SNAPSHOTS)
			return PGS_ERROR_CAPACITY;
		const uint32_t slot = snapshots_taken;
		if (!d_tex_snap[slot])
		{
			CUDA_TRY(cudaMalloc(&d_tex_snap[slot], size_t(max_planes) * VRAM_SIZE));
			if (graph_exec) { cudaGraphExecDestroy(graph_exec); graph_exec = nullptr; }
		}
		Op op = {};
		op.type = OP_SNAPSHOT;
		op.snap_slot = slot;
		int r = submit(op);
		if (r)
			return r;
		snapshots_taken++;
		return int(slot);
	}

	int copy_vram(const pgs_copy_desc *d)
	{
		Op op = {};
		op.type = OP_COPY;
		CopyParams &c = op.copy;
		uint64_t bb = d->bitbltbuf;
		c.sbp = field(bb, 0, 14); c.sbw = field(bb, 16, 6); c.spsm = field(bb, 24, 6);
		c.dbp = field(bb, 32, 14); c.dbw = field(bb, 48, 6); c.dpsm = field(bb, 56, 6);
		c.ssax = field(d->trxpos, 0, 11); c.ssay = field(d->trxpos, 16, 11);
		c.dsax = field(d->trxpos, 32, 11); c.dsay = field(d->trxpos, 48, 11);
		c.width = field(d->trxreg, 0, 12); c.height = field(d->trxreg, 32, 12);
		c.xdir = field(d->trxdir, 0, 2);
		c.invalidate_ss = num_planes > 1;
		if (c.width == 0 || c.height == 0 || (c.xdir != HOST_TO_LOCAL && c.xdir != LOCAL_TO_LOCAL))
			return PGS_OK;
		if (c.xdir == HOST_TO_LOCAL)
		{
			if (!d->host_data)
				return PGS_ERROR_INVALID_ARGUMENT;
			c.host_size = d->host_size;
			c.host_offset_qwords = d->host_offset / 8;
			size_t off;
			int r = arena_alloc(d->host_size, off);
			if (r)
				return r;
			memcpy(h_arena + off, d->host_data, d->host_size);
			// One host->device copy for a run of payloads placed back to back.
			if (pending_h2d_hi != off)
			{
				r = flush_pending_h2d();
				if (r)
					return r;
				pending_h2d_lo = off;
			}
			pending_h2d_hi = off + align_up(d->host_size, 256);
			h2d_bytes += d->host_size;
			op.copy_host_off = off;
		}
		return submit(op);
	}

	int update_palette(const pgs_palette_upload *u)
	{
		Op op = {};
		op.type = OP_CLUT;
		ClutParams &c = op.clut;
		uint64_t t = u->tex0;
		c.psm = uint32_t((t >> 20) & 0x3f);
		c.cbp = uint32_t((t >> 37) & 0x3fff);
		c.cpsm = uint32_t((t >> 51) & 0xf);
		c.csm = uint32_t((t >> 55) & 1);
		c.csa = uint32_t((t >> 56) & 0x1f);
		c.cbw = field(u->texclut, 0, 6);
		c.cou = field(u->texclut, 6, 6);
		c.cov = field(u->texclut, 12, 10);
		c.csm2_x_scale = u->csm2_x_scale;
		c.csm2_x_bias = u->csm2_x_bias;
		c.base_instance = u->base_instance % PGS_CLUT_INSTANCES;
		last_clut = u->target ? (u->target - 1u) % PGS_CLUT_INSTANCES : (last_clut + 1) % PGS_CLUT_INSTANCES;
		c.instance = last_clut;
		int r = submit(op);
		return r ? r : int(c.instance);
	}

	int set_super_sampling(uint32_t x, uint32_t y)
	{
		uint32_t planes = (x | y) ? 2u + (1u << (x + y)) : 1u;
		if (planes > max_planes)
			return PGS_ERROR_UNSUPPORTED;
		if (x > 2 || y > 3 || x > y)
			return PGS_ERROR_INVALID_ARGUMENT;
		rate_x = x;
		rate_y = y;
		num_planes = planes;
		if (max_planes > 1)
			CUDA_TRY(cudaMemsetAsync(d_vram + VRAM_SIZE, 0, size_t(max_planes - 1) * VRAM_SIZE, stream));
		build_phase_lut(x, y, h_phase_lut);
		CUDA_TRY(cudaMemcpyAsync(d_phase_lut, h_phase_lut, sizeof(h_phase_lut), cudaMemcpyHostToDevice, stream));
		CUDA_TRY(cudaStreamSynchronize(stream));
		return PGS_OK;
	}
	uint32_t h_phase_lut[PHASE_LUT_WORDS] = {};

	// A render pass instance that samples one per-sample texture at more than
	// one texel phase is taken for a blur kernel
	// (render_pass_instance_is_deduced_blur, gs/gs_renderer.cpp:1850-1884).
	// Blend demotion (gs/gs_renderer.cpp:2082-2091): 32 primitives per
	// coarse tile when the hack is on and every state of the pass blends.
	static uint32_t blend_demote_budget(const pgs_render_pass *rp)
	{
		if (!rp->blend_demote)
			return 0;
		for (uint32_t i = 0; i < rp->num_states; i++)
			if ((rp->states[i].blend_mode & BLEND_MODE_ABE_BIT) == 0)
				return 0;
		return 32;
	}

	// render_pass_instance_might_field_render (gs/gs_renderer.cpp:1888-1895):
	// an instance that ends above row 256 may be a field; taller ones are
	// taken as full frames that are downsampled later.
	static bool might_field_render(const PassOp &p, uint32_t instance)
	{
		const pgs_rp_instance &in = p.instances[instance];
		return !(in.base_y + int32_t(in.coarse_tiles_height << p.tile_size_log2) > 256);
	}

	static uint32_t blur_mask(const pgs_render_pass *rp)
	{
		if (rp->num_primitives > 64)
			return 0;
		uint32_t mask = 0;
		for (uint32_t inst = 0; inst < rp->num_instances; inst++)
		{
			uint32_t last = 0xffffffffu;
			int32_t phase[2] = { 0, 0 };
			for (uint32_t i = 0; i < rp->num_primitives; i++)
			{
				const pgs_primitive_attribute &pa = rp->prims[i];
				if (((pa.state >> STATE_VERTEX_RENDER_PASS_INSTANCE_OFFSET) & 7u) != inst || !(pa.tex & TEX_PER_SAMPLE_BIT))
					continue;
				if (pa.state & (1u << STATE_BIT_PERSPECTIVE))
					break;
				const uint32_t ti = pa.tex & TEX_TEXTURE_INDEX_MASK;
				const int32_t ph[2] = { int32_t(rp->attributes[3 * i].u) - rp->positions[3 * i].x,
				                        int32_t(rp->attributes[3 * i].v) - rp->positions[3 * i].y };
				if (last == ti)
				{
					if (ph[0] != phase[0] || ph[1] != phase[1])
					{
						mask |= 1u << inst;
						break;
					}
				}
				else
				{
					phase[0] = ph[0];
					phase[1] = ph[1];
				}
				last = ti;
			}
		}
		return mask;
	}

	// ------------------------------------------------------------------
	// Host->local uploads and CLUT loads wait in `deferred` until the next
	// operation that is not one of them, or anything else that touches the
	// stream or reads results (every entry point but copy_vram,
	// update_palette_cache and reserve_primitive_buffers flushes first), so
	// that a run of them goes out as one batched launch each, with one
	// host->device copy of their payloads.
	static bool deferrable(const Op &op)
	{
		return (op.type == OP_COPY && op.copy.xdir == HOST_TO_LOCAL) || op.type == OP_CLUT;
	}

	std::vector<Op> deferred;
	size_t pending_h2d_lo = 0, pending_h2d_hi = 0; // arena bytes not yet copied to the device
	int deferred_status = PGS_OK;

	int flush_pending_h2d()
	{
		if (pending_h2d_hi > pending_h2d_lo)
		{
			const size_t lo = pending_h2d_lo, size = pending_h2d_hi - pending_h2d_lo;
			pending_h2d_lo = pending_h2d_hi = 0;
			CUDA_TRY(cudaMemcpyAsync(d_arena + lo, h_arena + lo, size, cudaMemcpyHostToDevice, stream));
		}
		return PGS_OK;
	}

	int flush_deferred()
	{
		int r = flush_pending_h2d();
		for (size_t i = 0; r == PGS_OK && i < deferred.size();)
			r = execute_from(deferred, i, nullptr);
		deferred.clear();
		if (r && !deferred_status)
			deferred_status = r;
		return r;
	}

	// Set while an op submitted outside recording runs: nothing will run it
	// again, so it may work on its arena records in place.
	bool live_op = false;

	int submit(Op &op)
	{
		if (recording)
			ops.push_back(op);
		if (deferrable(op))
		{
			deferred.push_back(op);
			return deferred.size() >= 64 ? flush_deferred() : PGS_OK;
		}
		int r = flush_deferred();
		if (r)
			return r;
		live_op = !recording;
		r = execute(op);
		live_op = false;
		return r;
	}

	int ensure_masks(size_t words, size_t tiles)
	{
		if (words > masks_cap)
		{
			cudaFree(d_masks);
			size_t cap = std::max(words, masks_cap * 2);
			CUDA_TRY(cudaMalloc(&d_masks, cap * sizeof(uint32_t)));
			masks_cap = cap;
			if (graph_exec) { cudaGraphExecDestroy(graph_exec); graph_exec = nullptr; }
		}
		if (tiles > flags_cap)
		{
			cudaFree(d_flags);
			size_t cap = std::max(tiles, flags_cap * 2);
			CUDA_TRY(cudaMalloc(&d_flags, cap * sizeof(uint32_t)));
			flags_cap = cap;
			if (graph_exec) { cudaGraphExecDestroy(graph_exec); graph_exec = nullptr; }
		}
		return PGS_OK;
	}

	static uint32_t effective_z_psm(uint32_t color, uint32_t depth)
	{
		// deduce_effectice_z_psm (gs/gs_renderer.cpp:2147-2180).
		if (color == PSMCT32 || color == PSMCT24 || color == PSMCT16S)
		{
			if (depth == PSMCT32) return PSMZ32;
			if (depth == PSMCT24) return PSMZ24;
			if (depth == PSMCT16 || depth == PSMCT16S) return PSMZ16S;
		}
		else if (color == PSMZ32 || color == PSMZ24 || color == PSMZ16S)
		{
			if (depth == PSMZ32) return PSMCT32;
			if (depth == PSMZ24) return PSMCT24;
			if (depth == PSMZ16S || depth == PSMZ16) return PSMCT16S;
		}
		return depth;
	}

	// Shading launches: the super-sampled variant for tiles that need it, then
	// the single-sampled variant (ubershader.comp dispatched twice,
	// gs/gs_renderer.cpp:2395-2415).
	template <bool AA, bool MIP>
	void launch_shade(const PassParams &P, const DevInstance &I, uint32_t ns_log2, uint32_t grid,
	                  const uint32_t *masks, const uint32_t *summary)
	{
		if (I.rate_y_log2 != 0)
		{
			switch (ns_log2)
			{
			case 1: shade_kernel<2, true, AA, MIP><<<grid, 128, 0, stream>>>(P, I, masks, summary, d_flags); break;
			case 2: shade_kernel<4, true, AA, MIP><<<grid, 256, 0, stream>>>(P, I, masks, summary, d_flags); break;
			case 3: shade_kernel<8, true, AA, MIP><<<grid, 512, 0, stream>>>(P, I, masks, summary, d_flags); break;
			default: shade_kernel<16, true, AA, MIP><<<grid, 1024, 0, stream>>>(P, I, masks, summary, d_flags); break;
			}
			launch_counter++;
		}
		shade_kernel<1, false, AA, MIP><<<grid, 64, 0, stream>>>(P, I, masks, summary, d_flags);
		launch_counter++;
	}

	// Bins and shades one instance segment.  With `collect` set, a segment the
	// batched kernel can shade is only binned and returned as a work item.
	int run_instance(const PassParams &P, const PassOp &p, uint32_t inst_index, uint32_t lo, uint32_t count,
	                 ShadeItem *collect = nullptr, bool *collected = nullptr)
	{
		if (collected)
			*collected = false;
		const pgs_rp_instance &in = p.instances[inst_index];
		DevInstance I = {};
		uint32_t frame_lo = uint32_t(in.frame), zbuf_lo = uint32_t(in.zbuf);
		I.fb_base = field(frame_lo, 0, 9) * BLOCKS_PER_PAGE;
		I.fb_stride = field(frame_lo, 16, 6);
		I.fb_psm = field(frame_lo, 24, 6);
		I.zb_base = field(zbuf_lo, 0, 9) * BLOCKS_PER_PAGE;
		I.zb_psm = in.z_sensitive ? effective_z_psm(I.fb_psm, field(zbuf_lo, 24, 4) | 0x30u) : 0xffffffffu;
		I.base_x = in.base_x;
		I.base_y = in.base_y;
		I.tiles_w = in.coarse_tiles_width;
		I.tiles_h = in.coarse_tiles_height;
		I.rate_x_log2 = in.sampling_rate_x_log2;
		I.rate_y_log2 = in.sampling_rate_y_log2;
		I.preserve_samples = in.channel_shuffle && in.sampling_rate_y_log2 != 0;
		const bool field_render = p.field_aware && might_field_render(p, inst_index);
		I.snap_mask_y = -(1 << I.rate_y_log2);
		if (I.rate_y_log2 && field_render)
			I.snap_mask_y >>= 1;
		I.force_ss = field_render;
		I.blend_demote = p.blend_demote;
		I.instance = inst_index;
		I.prim_lo = lo;
		I.prim_count = count;
		I.mask_words = (count + 31) / 32;
		I.summary_words = (I.mask_words + 31) / 32;
		I.sub_w = I.tiles_w << (p.tile_size_log2 - 3);
		I.sub_h = I.tiles_h << (p.tile_size_log2 - 3);
		size_t tiles = size_t(I.tiles_w) * I.tiles_h;
		size_t subs = size_t(I.sub_w) * I.sub_h;
		if (tiles == 0 || count == 0)
			return PGS_OK;
		uint32_t ns_log2 = I.rate_x_log2 + I.rate_y_log2;
		if (I.rate_y_log2 > 3 || I.rate_x_log2 > 2 || ns_log2 > 4 || I.rate_x_log2 > I.rate_y_log2)
			return PGS_ERROR_INVALID_ARGUMENT;
		// Super-sampled shading touches planes 1 .. 1 + 2^ns_log2.
		if (I.rate_y_log2 != 0 && 2u + (1u << ns_log2) > num_planes)
			return PGS_ERROR_INVALID_ARGUMENT;
		size_t mask_words = subs * I.mask_words, summary_words = subs * I.summary_words;
		int r = ensure_masks(mask_words + summary_words, tiles);
		if (r)
			return r;
		uint32_t *d_sub_masks = d_masks, *d_sub_summary = d_masks + mask_words;
		{
			StageScope ts(this, PGS_TIMESTAMP_BINNING);
			CUDA_TRY(cudaMemsetAsync(d_masks, 0, (mask_words + summary_words) * sizeof(uint32_t), stream));
			CUDA_TRY(cudaMemsetAsync(d_flags, 0, tiles * sizeof(uint32_t), stream));
			bin_kernel<<<(count + 31) / 32, 32 * BIN_GROUP_WARPS, 0, stream>>>(P, I, d_sub_masks, d_sub_summary, d_flags);
			launch_counter++;
		}
		uint32_t grid = uint32_t(subs);
		if (collect && !p.has_mipmap && !p.has_ss_textures && ns_log2 <= BATCH_MAX_NS_LOG2 &&
		    (I.rate_y_log2 != 0 || ns_log2 == 0))
		{
			collect->P = P;
			collect->I = I;
			collect->masks = d_sub_masks;
			collect->summary = d_sub_summary;
			collect->flags = d_flags;
			collect->ns_log2 = I.rate_y_log2 != 0 ? ns_log2 : 0u;
			collect->aa = p.has_aa1;
			collect->units = uint32_t(subs) * (2u << collect->ns_log2);
			*collected = true;
			CUDA_TRY(cudaGetLastError());
			return PGS_OK;
		}
		if (shade_timing && !shade_started)
		{
			int r = record_timing_event(shade_ev[0]);
			if (r)
				return r;
			shade_started = true;
		}
		// Passes with mip levels or super-sampled textures take the AA-capable
		// variant too (three variants per rate).
		StageScope ts(this, PGS_TIMESTAMP_SHADING);
		if (p.has_mipmap || p.has_ss_textures)
			launch_shade<true, true>(P, I, ns_log2, grid, d_sub_masks, d_sub_summary);
		else if (p.has_aa1)
			launch_shade<true, false>(P, I, ns_log2, grid, d_sub_masks, d_sub_summary);
		else
			launch_shade<false, false>(P, I, ns_log2, grid, d_sub_masks, d_sub_summary);
		CUDA_TRY(cudaGetLastError());
		if (shade_timing)
			return record_timing_event(shade_ev[1]);
		return PGS_OK;
	}

	// Inside stream capture the event must be recorded as an external node so
	// that every graph launch records it; outside capture a plain record.
	int record_timing_event(cudaEvent_t ev)
	{
		cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
		CUDA_TRY(cudaStreamIsCapturing(stream, &cs));
		if (cs == cudaStreamCaptureStatusActive)
			CUDA_TRY(cudaEventRecordWithFlags(ev, stream, cudaEventRecordExternal));
		else
			CUDA_TRY(cudaEventRecord(ev, stream));
		return PGS_OK;
	}

	int execute(const Op &op)
	{
		switch (op.type)
		{
		case OP_COPY:
		{
			CopyParams c = op.copy;
			if (c.xdir == HOST_TO_LOCAL)
				c.host = d_arena + op.copy_host_off;
			else
			{
				CUDA_TRY(cudaMemcpyAsync(d_snapshot, d_vram, VRAM_SIZE, cudaMemcpyDeviceToDevice, stream));
				c.src_vram = d_snapshot;
			}
			StageScope ts(this, PGS_TIMESTAMP_COPY_VRAM);
			upload_kernel<<<dim3((c.width + 31) / 32, (c.height + 7) / 8), 256, 0, stream>>>(c, d_vram);
			launch_counter++;
			CUDA_TRY(cudaGetLastError());
			return PGS_OK;
		}
		case OP_CLUT:
		{
			StageScope ts(this, PGS_TIMESTAMP_PALETTE_UPDATE);
			clut_kernel<<<1, 256, 0, stream>>>(op.clut, d_vram, d_clut);
			launch_counter++;
			CUDA_TRY(cudaGetLastError());
			return PGS_OK;
		}
		case OP_PASS:
			return execute_pass(op.pass);
		case OP_SNAPSHOT:
			CUDA_TRY(cudaMemcpyAsync(d_tex_snap[op.snap_slot], d_vram, size_t(max_planes) * VRAM_SIZE,
			                         cudaMemcpyDeviceToDevice, stream));
			return PGS_OK;
		}
		return PGS_ERROR_INVALID_ARGUMENT;
	}

	// VRAM blocks (256 bytes) a host->local upload can write, one entry per
	// block-sized cell of its rectangle (a cell is one block whatever the
	// swizzle); false when the rectangle wraps the 2048 x 2048 address space.
	static bool upload_blocks(const CopyParams &c, std::vector<uint32_t> &out)
	{
		out.clear();
		if (c.dsax + c.width > 2048u || c.dsay + c.height > 2048u || c.width == 0 || c.height == 0)
			return false;
		const Layout L = psm_layout(c.dpsm);
		const uint32_t x1 = c.dsax + c.width - 1u, y1 = c.dsay + c.height - 1u;
		for (uint32_t cy = c.dsay >> L.bh; cy <= y1 >> L.bh; cy++)
			for (uint32_t cx = c.dsax >> L.bw; cx <= x1 >> L.bw; cx++)
			{
				const uint32_t x = std::max(cx << L.bw, c.dsax), y = std::max(cy << L.bh, c.dsay);
				const uint32_t a = swizzle_address(x, y, c.dbp, c.dbw, c.dpsm);
				const uint32_t byte = c.dpsm == PSMT4 ? a >> 1 : c.dpsm == PSMT8 ? a : psm_is_16bit(c.dpsm) ? a * 2u : a * 4u;
				out.push_back((byte >> 8) & (VRAM_SIZE / 256u - 1u));
			}
		return true;
	}

	// Blocks of each host->local upload of `ops`, by op index (filled on first use).
	std::vector<std::vector<uint32_t>> op_blocks;
	std::vector<uint8_t> op_blocks_state; // 0 unknown, 1 known, 2 not batchable

	// Runs list[i] and advances i.  Consecutive host->local uploads whose
	// destination pages do not overlap, and chains of CLUT loads, go in one
	// launch each (replays; the recording run executes one op at a time).
	int execute_from(const std::vector<Op> &list, size_t &i) { return execute_from(list, i, &op_blocks); }

	// blocks_cache: the block lists of `list` by index, kept across calls
	// (the recorded frame), or NULL to compute them each time.
	int execute_from(const std::vector<Op> &list, size_t &i, std::vector<std::vector<uint32_t>> *blocks_cache)
	{
		const Op &first = list[i];
		if (first.type == OP_COPY && first.copy.xdir == HOST_TO_LOCAL)
		{
			UploadBatch B;
			B.count = 0;
			uint32_t blocks = 0;
			size_t j = i;
			if (blocks_cache && blocks_cache->size() != list.size())
			{
				blocks_cache->assign(list.size(), {});
				op_blocks_state.assign(list.size(), 0);
			}
			std::vector<uint64_t> &used = batch_blocks;
			used.assign(VRAM_SIZE / 256u / 64u, 0);
			while (j < list.size() && B.count < UPLOAD_BATCH_MAX && list[j].type == OP_COPY &&
			       list[j].copy.xdir == HOST_TO_LOCAL)
			{
				const std::vector<uint32_t> *cells = &scratch_blocks;
				if (blocks_cache)
				{
					if (!op_blocks_state[j])
						op_blocks_state[j] = upload_blocks(list[j].copy, (*blocks_cache)[j]) ? 1 : 2;
					if (op_blocks_state[j] != 1)
						break;
					cells = &(*blocks_cache)[j];
				}
				else if (!upload_blocks(list[j].copy, scratch_blocks))
					break;
				bool overlap = false;
				for (uint32_t b : *cells)
					overlap = overlap || ((used[b >> 6] >> (b & 63u)) & 1u);
				if (overlap)
					break;
				for (uint32_t b : *cells)
					used[b >> 6] |= 1ull << (b & 63u);
				CopyParams c = list[j].copy;
				c.host = d_arena + list[j].copy_host_off;
				B.c[B.count] = c;
				B.block_start[B.count] = blocks;
				blocks += ((c.width + 31u) / 32u) * ((c.height + 7u) / 8u);
				B.count++;
				j++;
			}
			if (B.count >= 2)
			{
				B.block_start[B.count] = blocks;
				StageScope ts(this, PGS_TIMESTAMP_COPY_VRAM);
				upload_batch_kernel<<<blocks, 256, 0, stream>>>(B, d_vram);
				launch_counter++;
				CUDA_TRY(cudaGetLastError());
				i = j;
				return PGS_OK;
			}
		}
		else if (first.type == OP_CLUT && first.clut.instance != first.clut.base_instance)
		{
			ClutBatch B;
			B.count = 0;
			size_t j = i;
			while (j < list.size() && B.count < CLUT_BATCH_MAX && list[j].type == OP_CLUT)
			{
				const ClutParams &c = list[j].clut;
				bool ok = !B.count || (c.base_instance == B.c[B.count - 1].instance && c.instance != B.c[0].base_instance);
				for (uint32_t k = 0; ok && k < B.count; k++)
					ok = c.instance != B.c[k].instance;
				if (!ok)
					break;
				B.c[B.count++] = c;
				j++;
			}
			if (B.count >= 2)
			{
				StageScope ts(this, PGS_TIMESTAMP_PALETTE_UPDATE);
				clut_batch_kernel<<<B.count, 256, 0, stream>>>(B, d_vram, d_clut);
				launch_counter++;
				CUDA_TRY(cudaGetLastError());
				i = j;
				return PGS_OK;
			}
		}
		return execute(list[i++]);
	}

	// One bin + shade dispatch: primitives [lo, lo + count) of instance `inst`.
	// `cached_depth`: depth is read from a snapshot of VRAM taken just before
	// the dispatch (frame and depth buffer share memory; see alias_split).
	struct Segment
	{
		uint32_t inst, lo, count;
		bool cached_depth = false;
	};

	int execute_pass(const PassOp &p)
	{
		PassParams P;
		std::vector<Segment> segs;
		int r = begin_pass(p, P, segs);
		if (r)
			return r;
		for (const Segment &s : segs)
		{
			r = run_segment(P, p, s);
			if (r)
				return r;
		}
		return PGS_OK;
	}

	// A segment with cached depth snapshots all VRAM planes first and is
	// always shaded directly (never collected for batched shading).
	int run_segment(const PassParams &P, const PassOp &p, const Segment &s, ShadeItem *collect = nullptr,
	                bool *collected = nullptr)
	{
		if (!s.cached_depth)
			return run_instance(P, p, s.inst, s.lo, s.count, collect, collected);
		const size_t bytes = size_t(num_planes) * VRAM_SIZE;
		if (bytes > zcache_cap)
		{
			cudaFree(d_zcache);
			d_zcache = nullptr;
			zcache_cap = 0;
			CUDA_TRY(cudaMalloc(&d_zcache, bytes));
			zcache_cap = bytes;
		}
		CUDA_TRY(cudaMemcpyAsync(d_zcache, d_vram, bytes, cudaMemcpyDeviceToDevice, stream));
		PassParams Pc = P;
		Pc.zcache = d_zcache;
		if (collected)
			*collected = false;
		return run_instance(Pc, p, s.inst, s.lo, s.count);
	}

	// Frame and depth buffer at the same base (GSRenderer::dispatch_shading,
	// gs/gs_renderer.cpp:2534-2650): colour writes can land in depth read by
	// other tiles, so the segment is cut up -- primitives before the first
	// depth-sensitive one as usual; while primitives write depth, one
	// primitive per dispatch; after the last depth write, depth is read from
	// a snapshot retaken whenever a depth-tested sprite overlaps the area the
	// current dispatch already covers (dispatch_read_aliased_depth_passes,
	// :2418-2487); with no depth reads left, as usual.
	static void alias_split(const PassOp &p, const pgs_primitive_attribute *hp, const Segment &s,
	                        std::vector<Segment> &out)
	{
		const pgs_rp_instance &in = p.instances[s.inst];
		const uint32_t zmask = (1u << STATE_BIT_Z_TEST) | (1u << STATE_BIT_Z_WRITE);
		if (!in.z_sensitive || (uint32_t(in.frame) & 0x1ffu) != (uint32_t(in.zbuf) & 0x1ffu))
		{
			out.push_back(s);
			return;
		}
		const uint32_t end = s.lo + s.count;
		auto inst_of = [&](uint32_t i) { return (hp[i].state >> STATE_VERTEX_RENDER_PASS_INSTANCE_OFFSET) & 7u; };
		uint32_t first_zs = end, last_zs = 0, last_zw = 0;
		bool zwrite = false;
		for (uint32_t i = s.lo; i < end; i++)
		{
			if (inst_of(i) != s.inst)
				continue;
			const uint32_t st = hp[i].state;
			if (st & (1u << STATE_BIT_Z_WRITE))
			{
				zwrite = true;
				last_zw = i;
			}
			if (st & zmask)
			{
				first_zs = std::min(first_zs, i);
				last_zs = i;
			}
		}
		if (first_zs == end)
		{
			out.push_back(s);
			return;
		}
		if (first_zs > s.lo)
			out.push_back({ s.inst, s.lo, first_zs - s.lo, false });
		uint32_t next = first_zs;
		if (zwrite)
		{
			for (uint32_t i = first_zs; i <= last_zw; i++)
				if (inst_of(i) == s.inst)
					out.push_back({ s.inst, i, 1, false });
			next = last_zw + 1;
			if (next >= end)
				return;
			if (last_zs <= last_zw)
			{
				out.push_back({ s.inst, next, end - next, false });
				return;
			}
		}
		int32_t bb[4] = { INT32_MAX, INT32_MAX, INT32_MIN, INT32_MIN };
		for (uint32_t i = next; i < end; i++)
		{
			const uint32_t st = hp[i].state;
			if (inst_of(i) != s.inst || !(st & (1u << STATE_BIT_SPRITE)))
				continue;
			const int16_t *pb = hp[i].bb;
			const bool overlap = std::max<int32_t>(bb[0], pb[0]) <= std::min<int32_t>(bb[2], pb[2]) &&
			                     std::max<int32_t>(bb[1], pb[1]) <= std::min<int32_t>(bb[3], pb[3]) && (st & zmask);
			if (overlap)
			{
				if (i > next)
					out.push_back({ s.inst, next, i - next, true });
				next = i;
				bb[0] = pb[0]; bb[1] = pb[1]; bb[2] = pb[2]; bb[3] = pb[3];
			}
			else
			{
				bb[0] = std::min<int32_t>(bb[0], pb[0]);
				bb[1] = std::min<int32_t>(bb[1], pb[1]);
				bb[2] = std::max<int32_t>(bb[2], pb[2]);
				bb[3] = std::max<int32_t>(bb[3], pb[3]);
			}
		}
		if (next < end)
			out.push_back({ s.inst, next, end - next, true });
	}

	// Setup, single-sample heuristic and texture decode of a pass; `segs`
	// receives the instance segments to bin and shade in order.
	int begin_pass(const PassOp &p, PassParams &P, std::vector<Segment> &segs)
	{
		render_passes++;
		segs.clear();
		P = {};
		P.pos = reinterpret_cast<const pgs_vertex_position *>(d_arena + p.pos_off);
		P.attr = reinterpret_cast<const pgs_vertex_attribute *>(d_arena + p.attr_off);
		P.states = reinterpret_cast<const pgs_state_vector *>(d_arena + p.states_off);
		P.textures = reinterpret_cast<const pgs_texture_desc *>(d_arena + p.textures_off);
		P.tex_images = reinterpret_cast<const TexImage *>(d_arena + p.images_off);
		P.max_tex_levels = p.max_levels;
		P.rp_is_blur_mask = p.rp_is_blur_mask;
		P.force_linear_ss = 0;
		if (p.has_ss_textures && p.field_aware)
			for (uint32_t i = 0; i < p.num_instances; i++)
				P.force_linear_ss |= might_field_render(p, i) ? 1u : 0u;
		P.phase_lut = d_phase_lut;
		if (p.num_texels > texels_cap)
		{
			cudaFree(d_texels);
			d_texels = nullptr;
			size_t cap = std::max<size_t>(p.num_texels, texels_cap * 2);
			CUDA_TRY(cudaMalloc(&d_texels, cap * sizeof(uint32_t)));
			texels_cap = cap;
			if (graph_exec) { cudaGraphExecDestroy(graph_exec); graph_exec = nullptr; }
		}
		P.texels = d_texels;
		// Setup and the single-sample heuristic rewrite primitive words in
		// place: a recorded pass works on a copy so that its records stay as
		// recorded for the next replay; a pass run once works on its records.
		P.prims = live_op ? reinterpret_cast<pgs_primitive_attribute *>(d_arena + p.prim_off) : d_prims_work;
		P.setup = d_setup;
		P.tattr = d_tattr;
		P.num_prims = p.num_prims;
		P.num_states = std::max<uint32_t>(p.num_states, 1);
		P.num_textures = std::max<uint32_t>(p.num_textures, 1);
		P.tile_size_log2 = p.tile_size_log2;
		P.has_aa1 = p.has_aa1;
		P.has_scanmsk = p.has_scanmsk;
		P.has_ss_reference = num_planes > 1;
		P.vram = d_vram;
		P.num_snaps = p.num_snaps;
		for (uint32_t k = 0; k < p.num_snaps; k++)
		{
			P.snap_vram[k] = d_tex_snap[k];
			P.snap_limit[k] = p.snap_limit[k];
		}
		P.clut = d_clut;
		P.rcp_float_lut = d_rcp_float;
		P.unorm_lut = d_unorm_lut;
		P.error_flags = d_error;
		P.fragment_counter = d_frags;
		P.heuristic = d_heuristic;
		P.heuristic_action = d_heuristic_action;
		HeuristicParams H = {};
		heuristic_params(p, P.packed_z_shift, H);
		for (uint32_t i = 0; i < p.num_instances; i++)
		{
			P.opaque_fbmask[i] = p.instances[i].opaque_fbmask;
			P.setup_rate_x_log2 = std::max(P.setup_rate_x_log2, p.instances[i].sampling_rate_x_log2);
			P.setup_rate_y_log2 = std::max(P.setup_rate_y_log2, p.instances[i].sampling_rate_y_log2);
		}
		if (!live_op)
			CUDA_TRY(cudaMemcpyAsync(d_prims_work, d_arena + p.prim_off, size_t(p.num_prims) * sizeof(pgs_primitive_attribute),
			                         cudaMemcpyDeviceToDevice, stream));
		{
			StageScope ts(this, PGS_TIMESTAMP_TRIANGLE_SETUP);
			if (H.instance_mask)
				CUDA_TRY(cudaMemsetAsync(d_heuristic, 0, sizeof(SsHeuristic), stream));
			setup_kernel<<<(p.num_prims + 127) / 128, 128, 0, stream>>>(P);
			launch_counter++;
			if (H.instance_mask)
			{
				// Flush order: setup, heuristic, binning (gs/gs_renderer.cpp:3157-3170).
				single_sample_heuristic_kernel<<<dim3(256, p.num_instances), 1024, 0, stream>>>(P, H);
				heuristic_apply_kernel<<<(p.num_prims + 255) / 256, 256, 0, stream>>>(P);
				launch_counter += 2;
			}
		}
		if (p.num_textures && p.num_texels)
		{
			StageScope ts(this, PGS_TIMESTAMP_TEXTURE_UPLOAD);
			dim3 grid((p.max_texels + 255) / 256, p.num_textures, p.max_levels);
			texture_decode_kernel<<<grid, 256, 0, stream>>>(P);
			launch_counter++;
		}
		CUDA_TRY(cudaGetLastError());

		pass_segments(p, segs);
		return PGS_OK;
	}

	// Instance segments of a pass in execution order, cut up where the frame
	// and depth buffers alias.
	void pass_segments(const PassOp &p, std::vector<Segment> &segs) const
	{
		instance_segments(p, segs);
		const pgs_primitive_attribute *hp =
		    p.host_prims ? p.host_prims : reinterpret_cast<const pgs_primitive_attribute *>(h_arena + p.prim_off);
		bool any_alias = false;
		for (uint32_t i = 0; i < p.num_instances; i++)
			any_alias = any_alias || (p.instances[i].z_sensitive &&
			                          (uint32_t(p.instances[i].frame) & 0x1ffu) == (uint32_t(p.instances[i].zbuf) & 0x1ffu));
		if (!any_alias)
			return;
		std::vector<Segment> split;
		for (const Segment &s : segs)
			alias_split(p, hp, s, split);
		segs.swap(split);
	}

	void instance_segments(const PassOp &p, std::vector<Segment> &segs) const
	{
		segs.clear();
		if (p.num_instances == 1)
		{
			segs.push_back({ 0, 0, p.num_prims });
			return;
		}

		// Per-instance primitive ranges and hazard-ordered segments
		// (gs/gs_renderer.cpp:3190-3266).  The instance of each primitive is
		// read from the host copy of the records.
		const pgs_primitive_attribute *hp =
		    p.host_prims ? p.host_prims : reinterpret_cast<const pgs_primitive_attribute *>(h_arena + p.prim_off);
		uint8_t hazard[8] = {};
		bool any = instance_hazards(p, hazard);
		if (any)
		{
			uint32_t active = 0, active_h = 0, base = 0;
			for (uint32_t i = 0; i < p.num_prims; i++)
			{
				uint32_t inst = (hp[i].state >> STATE_VERTEX_RENDER_PASS_INSTANCE_OFFSET) & 7u;
				if (active_h & (1u << inst))
				{
					for (uint32_t b = 0; b < 8; b++)
						if (active & (1u << b))
							segs.push_back({ b, base, i - base });
					base = i;
					active = 0;
					active_h = 0;
				}
				active |= 1u << inst;
				active_h |= hazard[inst];
			}
			for (uint32_t b = 0; b < 8; b++)
				if (active & (1u << b))
					segs.push_back({ b, base, p.num_prims - base });
			return;
		}
		uint32_t lo[8], hi[8];
		for (int i = 0; i < 8; i++) { lo[i] = 0xffffffffu; hi[i] = 0; }
		for (uint32_t i = 0; i < p.num_prims; i++)
		{
			uint32_t inst = (hp[i].state >> STATE_VERTEX_RENDER_PASS_INSTANCE_OFFSET) & 7u;
			if (lo[inst] == 0xffffffffu) lo[inst] = i;
			hi[inst] = i;
		}
		for (uint32_t i = 0; i < p.num_instances; i++)
			if (lo[i] != 0xffffffffu)
				segs.push_back({ i, lo[i], hi[i] - lo[i] + 1 });
	}

	// Depth quantisation of the flat-primitive buckets per instance.  Triangle
	// setup buckets by Z >> (8, 16, 24) for Z16, Z24, Z32 (gs/gs_renderer.cpp:
	// 1914-1934); the heuristic walks 2^16 (2^8) values per bucket
	// (:1998-2030).  An instance that does not test Z counts as Z24.  A
	// format outside the four keeps the previous super-sampled instance's
	// parameters, as the reference's push constants do.
	static void heuristic_params(const PassOp &p, uint32_t &packed_z_shift, HeuristicParams &H)
	{
		packed_z_shift = 0;
		H = {};
		uint32_t zsb = 0, zs = 0, zmax = 0;
		for (uint32_t i = 0; i < p.num_instances; i++)
		{
			const pgs_rp_instance &in = p.instances[i];
			uint32_t depth_psm = in.z_sensitive ? (field(uint32_t(in.zbuf), 24, 4) | 0x30u) : PSMZ24;
			switch (depth_psm)
			{
			case PSMZ16S: case PSMZ16: packed_z_shift |= 1u << (4 * i); break;
			case PSMZ24: packed_z_shift |= 2u << (4 * i); break;
			case PSMZ32: packed_z_shift |= 3u << (4 * i); break;
			default: break;
			}
			if (in.sampling_rate_y_log2 == 0)
				continue;
			switch (depth_psm)
			{
			case PSMZ16S: case PSMZ16: zsb = 8; zs = 0; zmax = 0xffffu; break;
			case PSMZ24: zsb = 16; zs = 0; zmax = 0xffffffu; break;
			case PSMZ32: zsb = 16; zs = 8; zmax = 0xffffffffu; break;
			default: break;
			}
			H.z_shift_bucket[i] = zsb;
			H.z_shift[i] = zs;
			H.z_max[i] = zmax;
			H.instance_mask |= 1u << i;
		}
	}

	static bool instance_hazards(const PassOp &p, uint8_t *mask)
	{
		struct Range { uint32_t s, e; };
		auto range = [&](uint32_t base_block, int32_t x, int32_t y, uint32_t w, uint32_t h, uint32_t stride, uint32_t psm) {
			Layout L = psm_layout(psm);
			if (psm == PSMT4 || psm == PSMT8) stride >>= 1;
			uint32_t px0 = uint32_t(x) >> L.pw, px1 = (uint32_t(x) + w - 1) >> L.pw;
			uint32_t py0 = uint32_t(y) >> L.ph, py1 = (uint32_t(y) + h - 1) >> L.ph;
			uint32_t base = base_block / BLOCKS_PER_PAGE;
			return Range{ base + py0 * stride + px0, base + py1 * stride + px1 + ((base_block % BLOCKS_PER_PAGE) ? 1u : 0u) };
		};
		Range fb[8] = {}, zb[8] = {};
		uint32_t ts = p.tile_size_log2;
		for (uint32_t i = 0; i < p.num_instances; i++)
		{
			auto &in = p.instances[i];
			uint32_t f = uint32_t(in.frame), z = uint32_t(in.zbuf);
			fb[i] = range(field(f, 0, 9) * 32, in.base_x, in.base_y, in.coarse_tiles_width << ts, in.coarse_tiles_height << ts,
			              field(f, 16, 6), field(f, 24, 6));
			if (in.z_sensitive)
				zb[i] = range(field(z, 0, 9) * 32, in.base_x, in.base_y, in.coarse_tiles_width << ts,
				              in.coarse_tiles_height << ts, field(f, 16, 6), field(z, 24, 4));
		}
		auto ov = [](Range a, Range b) { return std::max(a.s, b.s) <= std::min(a.e, b.e); };
		bool any = false;
		for (uint32_t i = 0; i < p.num_instances; i++)
			for (uint32_t j = i + 1; j < p.num_instances; j++)
			{
				auto &a = p.instances[i], &b = p.instances[j];
				bool h = ov(fb[i], fb[j]) || (b.z_sensitive && ov(fb[i], zb[j])) || (a.z_sensitive && ov(fb[j], zb[i])) ||
				         (a.z_sensitive && b.z_sensitive && (a.z_write || b.z_write) && ov(zb[i], zb[j]));
				if (h)
				{
					mask[i] |= uint8_t(1u << j);
					mask[j] |= uint8_t(1u << i);
					any = true;
				}
			}
		return any;
	}

	// ------------------------------------------------------------------
	int read_vram(uint32_t plane, uint64_t off, uint64_t size, void *dst)
	{
		if (plane >= num_planes || off + size > VRAM_SIZE)
			return PGS_ERROR_INVALID_ARGUMENT;
		{
			StageScope ts(this, PGS_TIMESTAMP_READBACK);
			CUDA_TRY(cudaMemcpyAsync(dst, d_vram + size_t(plane) * VRAM_SIZE + off, size, cudaMemcpyDeviceToHost,
			                         stream));
		}
		CUDA_TRY(cudaStreamSynchronize(stream));
		d2h_bytes += size;
		total_launches += launch_counter;
		launch_counter = 0;
		if (!recording)
			arena_used = 0;
		return PGS_OK;
	}

	int read_vram_async(uint64_t off, uint64_t size, void *dst, uint64_t &ticket)
	{
		if (off + size > VRAM_SIZE)
			return PGS_ERROR_INVALID_ARGUMENT;
		// Oldest slot when all are busy: finish it first.
		Readback *slot = nullptr;
		for (auto &rb : readbacks)
			if (rb.ticket == 0) { slot = &rb; break; }
		if (!slot)
		{
			slot = &readbacks[0];
			for (auto &rb : readbacks)
				if (rb.ticket < slot->ticket) slot = &rb;
			int r = wait_ticket(slot->ticket);
			if (r)
				return r;
		}
		cudaPointerAttributes attr = {};
		bool pinned = cudaPointerGetAttributes(&attr, dst) == cudaSuccess && attr.type == cudaMemoryTypeHost;
		cudaGetLastError();
		void *target = dst;
		if (!pinned)
		{
			if (!slot->staging)
				CUDA_TRY(cudaMallocHost(&slot->staging, VRAM_SIZE));
			target = slot->staging;
		}
		{
			StageScope ts(this, PGS_TIMESTAMP_READBACK);
			CUDA_TRY(cudaMemcpyAsync(target, d_vram + off, size, cudaMemcpyDeviceToHost, stream));
		}
		CUDA_TRY(cudaEventRecord(slot->done, stream));
		slot->ticket = next_ticket++;
		slot->dst = pinned ? nullptr : dst;
		slot->size = size;
		d2h_bytes += size;
		total_launches += launch_counter;
		launch_counter = 0;
		ticket = slot->ticket;
		return PGS_OK;
	}

	int wait_ticket(uint64_t ticket)
	{
		for (auto &rb : readbacks)
		{
			if (rb.ticket != ticket)
				continue;
			CUDA_TRY(cudaEventSynchronize(rb.done));
			if (rb.dst)
				memcpy(rb.dst, rb.staging, rb.size);
			rb.ticket = 0;
			rb.dst = nullptr;
			return PGS_OK;
		}
		// Unknown or already waited for.
		return ticket && ticket < next_ticket ? PGS_OK : PGS_ERROR_INVALID_ARGUMENT;
	}

	int sample_circuit_device(const pgs_circuit_params &c, uint32_t *d_dst)
	{
		if (size_t(c.width) * c.height == 0)
			return PGS_OK;
		if (c.super_samples > 1 && 2u + c.super_samples > num_planes)
			return PGS_ERROR_INVALID_ARGUMENT;
		dim3 grid((c.width + 31) / 32, (c.height + 7) / 8);
		circuit_kernel<<<grid, 256, 0, stream>>>(c, d_vram, d_unorm_lut, d_dst);
		launch_counter++;
		CUDA_TRY(cudaGetLastError());
		return PGS_OK;
	}

	int sample_circuit(const pgs_circuit_params &c, void *dst)
	{
		size_t bytes = size_t(c.width) * c.height * 4u;
		if (bytes == 0)
			return PGS_OK;
		if (c.super_samples > 1 && 2u + c.super_samples > num_planes)
			return PGS_ERROR_INVALID_ARGUMENT;
		if (bytes > circuit_cap)
		{
			cudaFree(d_circuit);
			d_circuit = nullptr;
			circuit_cap = 0;
			CUDA_TRY(cudaMalloc(&d_circuit, bytes));
			circuit_cap = bytes;
		}
		dim3 grid((c.width + 31) / 32, (c.height + 7) / 8);
		circuit_kernel<<<grid, 256, 0, stream>>>(c, d_vram, d_unorm_lut, d_circuit);
		launch_counter++;
		CUDA_TRY(cudaGetLastError());
		CUDA_TRY(cudaMemcpyAsync(dst, d_circuit, bytes, cudaMemcpyDeviceToHost, stream));
		CUDA_TRY(cudaStreamSynchronize(stream));
		d2h_bytes += bytes;
		return PGS_OK;
	}

	// LOCAL->HOST read-out of a source rectangle, de-swizzled on the device:
	// only the rectangle's bytes cross to the host.
	int readback_rect(const pgs_copy_desc &d, void *dst, uint64_t dst_size)
	{
		ReadbackParams R = {};
		R.sbp = field(d.bitbltbuf, 0, 14);
		R.sbw = field(d.bitbltbuf, 16, 6);
		R.spsm = field(d.bitbltbuf, 24, 6);
		R.ssax = field(d.trxpos, 0, 11);
		R.ssay = field(d.trxpos, 16, 11);
		R.width = field(d.trxreg, 0, 12);
		R.height = field(d.trxreg, 32, 12);
		switch (R.spsm)
		{
		case PSMCT32: case PSMZ32: R.bytes_per_pixel = 4; break;
		case PSMCT24: case PSMZ24: R.bytes_per_pixel = 3; break;
		case PSMCT16: case PSMCT16S: case PSMZ16: case PSMZ16S: R.bytes_per_pixel = 2; break;
		case PSMT8: case PSMT8H: R.bytes_per_pixel = 1; break;
		default: return PGS_OK; // 4-bit formats: nothing to read out
		}
		R.size = uint64_t(R.width) * R.height * R.bytes_per_pixel;
		if (R.size == 0)
			return PGS_OK;
		if (!dst || dst_size < R.size)
			return PGS_ERROR_INVALID_ARGUMENT;
		if (R.size > readback_cap)
		{
			cudaFree(d_readback);
			d_readback = nullptr;
			readback_cap = 0;
			CUDA_TRY(cudaMalloc(&d_readback, R.size));
			readback_cap = R.size;
		}
		{
			StageScope ts(this, PGS_TIMESTAMP_READBACK);
			const uint64_t threads = (R.size + 15u) / 16u;
			readback_kernel<<<uint32_t((threads + 255u) / 256u), 256, 0, stream>>>(R, d_vram, d_readback);
			launch_counter++;
			CUDA_TRY(cudaGetLastError());
			CUDA_TRY(cudaMemcpyAsync(dst, d_readback, R.size, cudaMemcpyDeviceToHost, stream));
		}
		CUDA_TRY(cudaStreamSynchronize(stream));
		d2h_bytes += R.size;
		return PGS_OK;
	}

	static int ensure_image(DevImage &im, size_t pixels)
	{
		if (pixels * 4 <= im.cap)
			return PGS_OK;
		cudaFree(im.ptr);
		im.ptr = nullptr;
		im.cap = 0;
		CUDA_TRY(cudaMalloc(&im.ptr, pixels * 4));
		im.cap = pixels * 4;
		return PGS_OK;
	}

	// One vsync (pgs_merge_params): circuits, merge, EXTWRITE, deinterlace.
	int vsync(const pgs_merge_params &m, void *dst)
	{
		if (recording)
			return PGS_ERROR_UNSUPPORTED;
		StageScope ts(this, PGS_TIMESTAMP_VSYNC);
		const pgs_circuit_params *cp[2] = { &m.circuit[0], &m.circuit[1] };
		for (int i = 0; i < 2; i++)
		{
			const pgs_circuit_params &c = *cp[i];
			if (size_t(c.width) * c.height == 0)
				continue;
			if (c.width > 4096 || c.height > 4096)
				return PGS_ERROR_INVALID_ARGUMENT;
			int r = ensure_image(vs_circuit[i], size_t(c.width) * c.height);
			if (r)
				return r;
			r = sample_circuit_device(c, vs_circuit[i].ptr);
			if (r)
				return r;
		}
		auto grid_of = [](uint32_t w, uint32_t h) { return dim3((w + 31) / 32, (h + 7) / 8); };
		if (m.raw_circuit == 1 || m.raw_circuit == 2)
		{
			const pgs_circuit_params &c = *cp[m.raw_circuit - 1];
			size_t bytes = size_t(c.width) * c.height * 4;
			if (bytes)
				CUDA_TRY(cudaMemcpyAsync(dst, vs_circuit[m.raw_circuit - 1].ptr, bytes, cudaMemcpyDeviceToHost, stream));
			CUDA_TRY(cudaStreamSynchronize(stream));
			d2h_bytes += bytes;
			return PGS_OK;
		}
		if (m.width == 0 || m.height == 0)
			return PGS_OK;
		if (m.width > 4096 || m.height > 4096)
			return PGS_ERROR_INVALID_ARGUMENT;
		if ((m.draw_circuit1 && size_t(cp[0]->width) * cp[0]->height == 0) ||
		    (m.draw_circuit2 && size_t(cp[1]->width) * cp[1]->height == 0))
			return PGS_ERROR_INVALID_ARGUMENT;
		const size_t pixels = size_t(m.width) * m.height;
		int r = ensure_image(vs_merged, pixels);
		if (r)
			return r;
		merge_kernel<<<grid_of(m.width, m.height), 256, 0, stream>>>(m, vs_circuit[0].ptr, vs_circuit[1].ptr,
		                                                            vs_merged.ptr);
		launch_counter++;
		CUDA_TRY(cudaGetLastError());
		if (m.ext_write && m.ext_width && m.ext_height)
		{
			const uint32_t *src = vs_merged.ptr;
			uint32_t sw = m.width, sh = m.height;
			if (m.ext_source == 1 || m.ext_source == 2)
			{
				const int ci = m.ext_source == 1 ? 1 : 0;
				if (size_t(cp[ci]->width) * cp[ci]->height == 0)
					return PGS_ERROR_INVALID_ARGUMENT;
				src = vs_circuit[ci].ptr;
				sw = cp[ci]->width;
				sh = cp[ci]->height;
			}
			if (m.ext_width > 4096 || m.ext_height > 4096)
				return PGS_ERROR_INVALID_ARGUMENT;
			extwrite_kernel<<<grid_of(m.ext_width, m.ext_height), 256, 0, stream>>>(m, src, sw, sh, d_unorm_lut, d_vram,
			                                                                      num_planes > 1 ? 1u : 0u);
			launch_counter++;
			CUDA_TRY(cudaGetLastError());
		}
		if (!m.deinterlace)
		{
			for (bool &v : vs_field_valid)
				v = false;
			CUDA_TRY(cudaMemcpyAsync(dst, vs_merged.ptr, pixels * 4, cudaMemcpyDeviceToHost, stream));
			CUDA_TRY(cudaStreamSynchronize(stream));
			d2h_bytes += pixels * 4;
			return PGS_OK;
		}
		// Field history: the new merged image becomes slot 0 and the others
		// move down; holes of the first frames take the newest fields
		// (:5015-5030).  A size change starts the history over.
		if (m.width != vs_field_w || m.height != vs_field_h)
		{
			for (bool &v : vs_field_valid)
				v = false;
			vs_field_w = m.width;
			vs_field_h = m.height;
		}
		std::swap(vs_fields[3], vs_fields[2]);
		std::swap(vs_fields[2], vs_fields[1]);
		std::swap(vs_fields[1], vs_fields[0]);
		std::swap(vs_fields[0], vs_merged);
		vs_field_valid[3] = vs_field_valid[2];
		vs_field_valid[2] = vs_field_valid[1];
		vs_field_valid[1] = vs_field_valid[0];
		vs_field_valid[0] = true;
		const int fill_from[4] = { 0, 0, 0, 1 };
		for (int i = 1; i < 4; i++)
		{
			if (vs_field_valid[i])
				continue;
			r = ensure_image(vs_fields[i], pixels);
			if (r)
				return r;
			CUDA_TRY(cudaMemcpyAsync(vs_fields[i].ptr, vs_fields[fill_from[i]].ptr, pixels * 4, cudaMemcpyDeviceToDevice,
			                         stream));
			vs_field_valid[i] = true;
		}
		r = ensure_image(vs_out, pixels * 2);
		if (r)
			return r;
		weave_kernel<<<grid_of(m.width, 2 * m.height), 256, 0, stream>>>(vs_fields[0].ptr, vs_fields[1].ptr,
		                                                                  vs_fields[2].ptr, vs_fields[3].ptr, m.width,
		                                                                  m.height, m.phase & 1u, d_unorm_lut, vs_out.ptr);
		launch_counter++;
		CUDA_TRY(cudaGetLastError());
		CUDA_TRY(cudaMemcpyAsync(dst, vs_out.ptr, pixels * 8, cudaMemcpyDeviceToHost, stream));
		CUDA_TRY(cudaStreamSynchronize(stream));
		d2h_bytes += pixels * 8;
		return PGS_OK;
	}

	int write_vram(uint64_t off, uint64_t size, const void *src)
	{
		if (off + size > VRAM_SIZE)
			return PGS_ERROR_INVALID_ARGUMENT;
		{
			StageScope ts(this, PGS_TIMESTAMP_SYNC_HOST_TO_VRAM);
			CUDA_TRY(cudaMemcpyAsync(d_vram + off, src, size, cudaMemcpyHostToDevice, stream));
			if (num_planes > 1)
				CUDA_TRY(cudaMemsetAsync(d_vram + VRAM_SIZE + off, 0, size, stream));
		}
		CUDA_TRY(cudaStreamSynchronize(stream));
		return PGS_OK;
	}

	int flush_submit()
	{
		return PGS_OK;
	}

	int get_error(uint32_t *flags)
	{
		uint32_t f = 0;
		CUDA_TRY(cudaMemcpyAsync(&f, d_error, sizeof(f), cudaMemcpyDeviceToHost, stream));
		CUDA_TRY(cudaStreamSynchronize(stream));
		if (flags)
			*flags = f;
		return f ? PGS_ERROR_DEVICE_FLAG : PGS_OK;
	}

	// ------------------------------------------------------------------
	int begin_record()
	{
		CUDA_TRY(cudaStreamSynchronize(stream));
		if (graph_exec)
		{
			cudaGraphExecDestroy(graph_exec);
			graph_exec = nullptr;
		}
		ops.clear();
		op_blocks.clear();
		op_blocks_state.clear();
		arena_used = 0;
		size_t vbytes = size_t(num_planes) * VRAM_SIZE;
		cudaFree(d_reset_vram);
		cudaFree(d_reset_clut);
		d_reset_vram = nullptr;
		d_reset_clut = nullptr;
		CUDA_TRY(cudaMalloc(&d_reset_vram, vbytes));
		CUDA_TRY(cudaMalloc(&d_reset_clut, size_t(PGS_CLUT_INSTANCES) * PGS_CLUT_SIZE_BYTES));
		CUDA_TRY(cudaMemcpyAsync(d_reset_vram, d_vram, vbytes, cudaMemcpyDeviceToDevice, stream));
		CUDA_TRY(cudaMemcpyAsync(d_reset_clut, d_clut, size_t(PGS_CLUT_INSTANCES) * PGS_CLUT_SIZE_BYTES,
		                         cudaMemcpyDeviceToDevice, stream));
		reset_planes = num_planes;
		recording = true;
		return PGS_OK;
	}

	int end_record()
	{
		recording = false;
		CUDA_TRY(cudaStreamSynchronize(stream));
		return PGS_OK;
	}

	int replay_once(bool reset)
	{
		launch_counter = 0;
		shade_started = false;
		if (reset && d_reset_vram)
		{
			CUDA_TRY(cudaMemcpyAsync(d_vram, d_reset_vram, size_t(reset_planes) * VRAM_SIZE, cudaMemcpyDeviceToDevice, stream));
			CUDA_TRY(cudaMemcpyAsync(d_clut, d_reset_clut, size_t(PGS_CLUT_INSTANCES) * PGS_CLUT_SIZE_BYTES,
			                         cudaMemcpyDeviceToDevice, stream));
		}
		for (size_t i = 0; i < ops.size();)
		{
			int r = execute_from(ops, i);
			if (r)
				return r;
		}
		launches_per_replay = launch_counter;
		return PGS_OK;
	}

	int replay(uint32_t count, bool reset, bool use_graph)
	{
		if (!use_graph)
		{
			for (uint32_t i = 0; i < count; i++)
			{
				int r = replay_once(reset);
				if (r)
					return r;
			}
			return PGS_OK;
		}
		if (!graph_exec)
		{
			// Make sure scratch buffers are sized before capture.
			int r = replay_once(reset);
			if (r)
				return r;
			CUDA_TRY(cudaStreamSynchronize(stream));
			cudaGraph_t graph;
			CUDA_TRY(cudaStreamBeginCapture(stream, cudaStreamCaptureModeThreadLocal));
			r = replay_once(reset);
			cudaError_t e = cudaStreamEndCapture(stream, &graph);
			if (r)
				return r;
			if (e != cudaSuccess)
				return PGS_ERROR_CUDA;
			CUDA_TRY(cudaGraphInstantiate(&graph_exec, graph, 0));
			cudaGraphDestroy(graph);
		}
		for (uint32_t i = 0; i < count; i++)
			CUDA_TRY(cudaGraphLaunch(graph_exec, stream));
		total_launches += uint64_t(count) * launches_per_replay;
		return PGS_OK;
	}
};

// ---------------------------------------------------------------------------
// Batched replay of many recorded command streams (one CudaBackend each).
//
// A round takes every stream one render pass further: the stream's transfers
// and CLUT loads before that pass, its setup / heuristic / texture decode, and
// the binning of its next instance segment run as one branch per stream; the
// branches join and a single persistent launch shades all collected segments.
// Streams with more instance segments continue in further sub-rounds.  The
// whole schedule is captured as one CUDA graph.
struct BatchEngine
{
	int device = 0;
	int sm_count = 0;
	cudaStream_t master = nullptr;
	cudaEvent_t fork_ev = nullptr;
	std::vector<CudaBackend *> streams;
	std::vector<cudaEvent_t> join_ev;

	// Work items of every sub-round, in schedule order.
	ShadeItem *h_items = nullptr, *d_items = nullptr;
	size_t items_cap = 0;
	uint32_t *d_counters = nullptr;
	size_t counters_cap = 0;
	size_t n_items = 0, n_launches = 0;

	// Tuning: persistent CTA size and CTAs per SM.
	uint32_t block = 256, ctas_per_sm = 4;
	bool largest_first = true;
	uint32_t solo_min_prims = 0;
	std::vector<bool> solo; // per stream, decided at the start of a run

	cudaGraphExec_t exec = nullptr;
	uint32_t launches_per_replay = 0;

	struct Cursor
	{
		size_t op = 0;
		const PassOp *pass = nullptr;
		PassParams P;
		std::vector<CudaBackend::Segment> segs;
		size_t seg = 0;
	};

	int init(int dev)
	{
		device = dev;
		CUDA_TRY(cudaSetDevice(device));
		CUDA_TRY(cudaDeviceGetAttribute(&sm_count, cudaDevAttrMultiProcessorCount, device));
		CUDA_TRY(cudaStreamCreateWithFlags(&master, cudaStreamNonBlocking));
		CUDA_TRY(cudaEventCreateWithFlags(&fork_ev, cudaEventDisableTiming));
		return PGS_OK;
	}

	void destroy()
	{
		cudaSetDevice(device);
		if (master)
			cudaStreamSynchronize(master);
		if (exec)
			cudaGraphExecDestroy(exec);
		for (cudaEvent_t e : join_ev)
			cudaEventDestroy(e);
		if (fork_ev)
			cudaEventDestroy(fork_ev);
		cudaFreeHost(h_items);
		cudaFree(d_items);
		cudaFree(d_counters);
		if (master)
			cudaStreamDestroy(master);
	}

	int add(CudaBackend *b)
	{
		if (b->device != device || b->ops.empty() || !b->d_reset_vram)
			return PGS_ERROR_INVALID_ARGUMENT;
		cudaEvent_t e;
		CUDA_TRY(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
		streams.push_back(b);
		join_ev.push_back(e);
		invalidate();
		return PGS_OK;
	}

	void invalidate()
	{
		if (exec)
		{
			cudaGraphExecDestroy(exec);
			exec = nullptr;
		}
	}

	// Round barriers involve the batched streams only; `all` includes the
	// solo streams (start and end of a run).
	int fork(bool all = false)
	{
		CUDA_TRY(cudaEventRecord(fork_ev, master));
		for (size_t i = 0; i < streams.size(); i++)
			if (all || !solo[i])
				CUDA_TRY(cudaStreamWaitEvent(streams[i]->stream, fork_ev, 0));
		return PGS_OK;
	}

	int join(bool all = false)
	{
		for (size_t i = 0; i < streams.size(); i++)
		{
			if (!all && solo[i])
				continue;
			CUDA_TRY(cudaEventRecord(join_ev[i], streams[i]->stream));
			CUDA_TRY(cudaStreamWaitEvent(master, join_ev[i], 0));
		}
		return PGS_OK;
	}

	static uint64_t frame_prims(const CudaBackend *b)
	{
		uint64_t n = 0;
		for (const Op &op : b->ops)
			if (op.type == OP_PASS)
				n += op.pass.num_prims;
		return n;
	}

	template <int BLOCK>
	int launch(size_t first, size_t count, uint32_t units, uint32_t counter)
	{
		uint32_t grid = std::max<uint32_t>(1u, std::min<uint32_t>(uint32_t(sm_count) * ctas_per_sm,
		                                                          (units + BLOCK / 32 - 1) / (BLOCK / 32)));
		batch_shade_kernel<BLOCK><<<grid, BLOCK, 0, master>>>(d_items + first, uint32_t(count), units,
		                                                      d_counters + counter);
		CUDA_TRY(cudaGetLastError());
		return PGS_OK;
	}

	// One pass over the schedule, launched (or captured) on the master stream
	// and the streams' own streams.
	int run(bool reset)
	{
		// An eager run rewrites the pinned item table, which an earlier run's
		// copies may still read.
		cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
		CUDA_TRY(cudaStreamIsCapturing(master, &cs));
		if (cs == cudaStreamCaptureStatusNone)
			CUDA_TRY(cudaStreamSynchronize(master));
		std::vector<Cursor> cur(streams.size());
		std::vector<ShadeItem> round_items;
		n_items = 0;
		n_launches = 0;
		uint32_t kernels = 0;
		for (CudaBackend *b : streams)
		{
			b->launch_counter = 0;
			b->shade_started = false;
		}
		if (counters_cap)
			CUDA_TRY(cudaMemsetAsync(d_counters, 0, counters_cap * sizeof(uint32_t), master));
		solo.assign(streams.size(), false);
		for (size_t s = 0; s < streams.size(); s++)
			solo[s] = solo_min_prims && frame_prims(streams[s]) >= solo_min_prims;
		int r = fork(true);
		if (r)
			return r;
		if (reset)
			for (CudaBackend *b : streams)
			{
				CUDA_TRY(cudaMemcpyAsync(b->d_vram, b->d_reset_vram, size_t(b->reset_planes) * VRAM_SIZE,
				                         cudaMemcpyDeviceToDevice, b->stream));
				CUDA_TRY(cudaMemcpyAsync(b->d_clut, b->d_reset_clut, size_t(PGS_CLUT_INSTANCES) * PGS_CLUT_SIZE_BYTES,
				                         cudaMemcpyDeviceToDevice, b->stream));
			}
		// Solo streams: the whole frame on the stream's own CUDA stream.
		for (size_t s = 0; s < streams.size(); s++)
		{
			if (!solo[s])
				continue;
			for (size_t i = 0; i < streams[s]->ops.size();)
			{
				r = streams[s]->execute_from(streams[s]->ops, i);
				if (r)
					return r;
			}
			cur[s].op = streams[s]->ops.size();
		}
		for (;;)
		{
			// Round: every stream up to and including the start of its next pass.
			bool any = false;
			for (size_t s = 0; s < streams.size(); s++)
			{
				if (solo[s])
					continue;
				CudaBackend *b = streams[s];
				Cursor &c = cur[s];
				c.pass = nullptr;
				c.segs.clear();
				c.seg = 0;
				while (c.op < b->ops.size() && b->ops[c.op].type != OP_PASS)
				{
					r = b->execute_from(b->ops, c.op);
					if (r)
						return r;
				}
				if (c.op < b->ops.size())
				{
					c.pass = &b->ops[c.op++].pass;
					r = b->begin_pass(*c.pass, c.P, c.segs);
					if (r)
						return r;
					any = true;
				}
			}
			if (!any)
				break;
			// Sub-rounds: one instance segment of every stream that has one.
			for (;;)
			{
				size_t first = n_items;
				round_items.clear();
				bool more = false;
				for (size_t s = 0; s < streams.size(); s++)
				{
					Cursor &c = cur[s];
					if (c.seg >= c.segs.size())
						continue;
					more = true;
					const CudaBackend::Segment &g = c.segs[c.seg++];
					ShadeItem item;
					bool collected = false;
					r = streams[s]->run_segment(c.P, *c.pass, g, &item, &collected);
					if (r)
						return r;
					if (collected && item.units)
					{
						if (n_items >= items_cap)
							return PGS_ERROR_CAPACITY;
						round_items.push_back(item);
						n_items++;
					}
				}
				if (!more)
					break;
				r = join();
				if (r)
					return r;
				if (n_items > first)
				{
					{
						if (n_launches >= counters_cap)
							return PGS_ERROR_CAPACITY;
						size_t count = n_items - first;
						if (largest_first)
							std::stable_sort(round_items.begin(), round_items.end(),
							                 [](const ShadeItem &a, const ShadeItem &b) { return a.units > b.units; });
						uint32_t units = 0;
						for (ShadeItem &x : round_items)
						{
							x.unit_base = units;
							units += x.units;
						}
						ShadeItem *it = h_items + first;
						memcpy(it, round_items.data(), count * sizeof(ShadeItem));
						CUDA_TRY(cudaMemcpyAsync(d_items + first, it, count * sizeof(ShadeItem), cudaMemcpyHostToDevice,
						                         master));
						switch (block)
						{
						case 128: r = launch<128>(first, count, units, uint32_t(n_launches)); break;
						case 512: r = launch<512>(first, count, units, uint32_t(n_launches)); break;
						default: r = launch<256>(first, count, units, uint32_t(n_launches)); break;
						}
						if (r)
							return r;
						kernels++;
					}
					n_launches++;
				}
				r = fork();
				if (r)
					return r;
			}
		}
		// Operations after the last pass of each stream.
		for (size_t s = 0; s < streams.size(); s++)
			while (cur[s].op < streams[s]->ops.size())
			{
				r = streams[s]->execute_from(streams[s]->ops, cur[s].op);
				if (r)
					return r;
			}
		r = join(true);
		if (r)
			return r;
		uint32_t total = kernels;
		for (CudaBackend *b : streams)
			total += b->launch_counter;
		launches_per_replay = total;
		return PGS_OK;
	}

	// Upper bounds of work items (every instance segment) and batched launches
	// (per round, the most segments any stream's pass has) from the recorded
	// operations alone, and buffers of that size.
	int size_buffers()
	{
		size_t items = 0, launches = 0;
		std::vector<std::vector<size_t>> per_stream(streams.size());
		std::vector<CudaBackend::Segment> segs;
		size_t rounds = 0;
		for (size_t s = 0; s < streams.size(); s++)
		{
			for (const Op &op : streams[s]->ops)
				if (op.type == OP_PASS)
				{
					streams[s]->pass_segments(op.pass, segs);
					per_stream[s].push_back(segs.size());
					items += segs.size();
				}
			rounds = std::max(rounds, per_stream[s].size());
		}
		for (size_t j = 0; j < rounds; j++)
		{
			size_t m = 0;
			for (auto &v : per_stream)
				if (j < v.size())
					m = std::max(m, v[j]);
			launches += m;
		}
		items = std::max<size_t>(items, 1);
		launches = std::max<size_t>(launches, 1);
		if (items > items_cap)
		{
			cudaFreeHost(h_items);
			cudaFree(d_items);
			h_items = nullptr;
			d_items = nullptr;
			items_cap = 0;
			CUDA_TRY(cudaMallocHost(&h_items, items * sizeof(ShadeItem)));
			CUDA_TRY(cudaMalloc(&d_items, items * sizeof(ShadeItem)));
			items_cap = items;
		}
		if (launches > counters_cap)
		{
			cudaFree(d_counters);
			d_counters = nullptr;
			counters_cap = 0;
			CUDA_TRY(cudaMalloc(&d_counters, launches * sizeof(uint32_t)));
			counters_cap = launches;
		}
		return PGS_OK;
	}

	int replay(uint32_t count, bool reset, bool use_graph)
	{
		if (streams.empty())
			return PGS_ERROR_INVALID_ARGUMENT;
		CUDA_TRY(cudaSetDevice(device));
		int r = size_buffers();
		if (r)
			return r;
		if (!use_graph)
		{
			for (uint32_t i = 0; r == PGS_OK && i < count; i++)
				r = run(reset);
			return r;
		}
		if (!exec)
		{
			if (count == 0)
				return PGS_OK;
			// The first replay runs eagerly: it sizes every stream's scratch
			// buffers, which must not be allocated during capture.
			r = run(reset);
			if (r)
				return r;
			count--;
			for (CudaBackend *b : streams)
				CUDA_TRY(cudaStreamSynchronize(b->stream));
			CUDA_TRY(cudaStreamSynchronize(master));
			cudaGraph_t graph;
			CUDA_TRY(cudaStreamBeginCapture(master, cudaStreamCaptureModeThreadLocal));
			r = run(reset);
			cudaError_t e = cudaStreamEndCapture(master, &graph);
			if (r)
				return r;
			if (e != cudaSuccess)
				return PGS_ERROR_CUDA;
			CUDA_TRY(cudaGraphInstantiate(&exec, graph, 0));
			cudaGraphDestroy(graph);
		}
		for (uint32_t i = 0; i < count; i++)
			CUDA_TRY(cudaGraphLaunch(exec, master));
		return PGS_OK;
	}
};

// ---------------------------------------------------------------------------
// pgs_backend_ops table.
// Every entry point makes the backend's device current for the calling
// thread: frontends of different streams may run on different host threads.
// The backend with its device current and its deferred uploads and CLUT
// loads issued: every entry point that may touch the stream or read results.
CudaBackend *B(void *s)
{
	CudaBackend *b = static_cast<CudaBackend *>(s);
	cudaSetDevice(b->device);
	b->flush_deferred();
	return b;
}

// Entry points that may leave uploads and CLUT loads deferred.
CudaBackend *B_defer(void *s)
{
	CudaBackend *b = static_cast<CudaBackend *>(s);
	cudaSetDevice(b->device);
	return b;
}

void c_destroy(void *self)
{
	if (!self) return;
	B(self)->destroy();
	delete B(self);
}
int c_reserve(void *self, uint32_t n, pgs_vertex_position **p, pgs_vertex_attribute **a, pgs_primitive_attribute **pr)
{
	// Handing out the staging buffers touches neither VRAM nor the stream.
	return B_defer(self)->reserve(n, p, a, pr);
}
int c_flush_rendering(void *self, const pgs_render_pass *rp) { return B(self)->flush_rendering(rp); }
int c_copy(void *self, const pgs_copy_desc *d) { return d ? B_defer(self)->copy_vram(d) : PGS_ERROR_INVALID_ARGUMENT; }
int c_palette(void *self, const pgs_palette_upload *u) { return u ? B_defer(self)->update_palette(u) : PGS_ERROR_INVALID_ARGUMENT; }
int c_set_ss(void *self, uint32_t x, uint32_t y) { return B(self)->set_super_sampling(x, y); }
int c_submit(void *self)
{
	CudaBackend *b = B(self);
	const int r = b->deferred_status;
	b->deferred_status = PGS_OK;
	return r ? r : b->flush_submit();
}
int c_read(void *self, uint32_t plane, uint64_t off, uint64_t size, void *dst)
{
	return dst ? B(self)->read_vram(plane, off, size, dst) : PGS_ERROR_INVALID_ARGUMENT;
}
int c_write(void *self, uint64_t off, uint64_t size, const void *src)
{
	return src ? B(self)->write_vram(off, size, src) : PGS_ERROR_INVALID_ARGUMENT;
}
int c_error(void *self, uint32_t *flags) { return B(self)->get_error(flags); }
int c_read_async(void *self, uint64_t off, uint64_t size, void *dst, uint64_t *ticket)
{
	return dst && ticket ? B(self)->read_vram_async(off, size, dst, *ticket) : PGS_ERROR_INVALID_ARGUMENT;
}
int c_wait(void *self, uint64_t ticket) { return B(self)->wait_ticket(ticket); }
int c_circuit(void *self, const pgs_circuit_params *c, void *dst)
{
	return c && dst ? B(self)->sample_circuit(*c, dst) : PGS_ERROR_INVALID_ARGUMENT;
}
static int c_vsync(void *self, const pgs_merge_params *m, void *dst)
{
	return m && dst ? B(self)->vsync(*m, dst) : PGS_ERROR_INVALID_ARGUMENT;
}
static int c_timestamps(void *self, int enable, double *totals) { return B(self)->timestamps(enable, totals); }
static int c_snapshot(void *self) { return B(self)->snapshot_vram(); }
static int c_readback(void *self, const pgs_copy_desc *d, void *dst, uint64_t size)
{
	return d ? B(self)->readback_rect(*d, dst, size) : PGS_ERROR_INVALID_ARGUMENT;
}

const pgs_backend_ops CUDA_OPS = {
	PGS_ABI_VERSION, c_destroy, c_reserve, c_flush_rendering, c_copy, c_palette, c_set_ss, c_submit, c_read, c_write, c_error,
	c_read_async, c_wait, c_circuit, c_vsync, c_timestamps, c_snapshot, c_readback,
};

// ---------------------------------------------------------------------------
// Allocation-free local->local copy.  The staging area is a file-scope device
// array; host code only ever uses the address cudaGetSymbolAddress returns.
static __device__ __align__(256) uint32_t g_noalloc_copy_scratch[PGS_NOALLOC_COPY_MAX_PIXELS];

// Set-up cache: the array's device address per CUDA context.  A context that
// is destroyed and created again (cudaDeviceReset, or a host framework that
// resets the device) loads the module again and the array can move, so the
// key is the context's process-unique ID (cuCtxGetId), not the device number.
constexpr int NOALLOC_MAX_CONTEXTS = 64;
std::mutex g_noalloc_mutex;
struct NoallocSlot
{
	unsigned long long ctx_id;
	uint32_t *ptr;
};
NoallocSlot g_noalloc_slots[NOALLOC_MAX_CONTEXTS] = {};
int g_noalloc_num_slots = 0;

// Pass 1: read every source pixel of the rectangle into the staging array.
__global__ void __launch_bounds__(256) noalloc_gather_kernel(CopyParams C, const uint8_t *vram, uint32_t *staging)
{
	uint32_t x = blockIdx.x * 32u + (threadIdx.x & 31u);
	uint32_t y = blockIdx.y * 8u + (threadIdx.x >> 5);
	if (x >= C.width || y >= C.height)
		return;
	uint32_t sx = (x + C.ssax) & 2047u, sy = (y + C.ssay) & 2047u;
	staging[y * C.width + x] = read_pixel(vram, C.spsm, swizzle_address(sx, sy, C.sbp, C.sbw, C.spsm));
}

// Pass 2: write the destination exactly as upload_kernel does for local copies.
__global__ void __launch_bounds__(256) noalloc_scatter_kernel(CopyParams C, uint8_t *vram, const uint32_t *staging)
{
	uint32_t x = blockIdx.x * 32u + (threadIdx.x & 31u);
	uint32_t y = blockIdx.y * 8u + (threadIdx.x >> 5);
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
	write_pixel(vram, C.dpsm, swizzle_address(dx, dy, C.dbp, C.dbw, C.dpsm), staging[y * C.width + x],
	            C.invalidate_ss != 0);
}

// Set-up, once per CUDA context: the device address of the staging array,
// looked up with that context current.  cuCtxGetCurrent / cuCtxGetId come
// through the runtime's driver entry points (no link against libcuda).
int noalloc_scratch(uint32_t **out)
{
	using CtxGetCurrent = int (*)(void **);
	using CtxGetId = int (*)(void *, unsigned long long *);
	static CtxGetCurrent get_current = nullptr;
	static CtxGetId get_id = nullptr;
	int dev = 0;
	if (cudaGetDevice(&dev) != cudaSuccess)
		return PGS_ERROR_NO_DEVICE;
	std::lock_guard<std::mutex> lock(g_noalloc_mutex);
	if (!get_current || !get_id)
	{
		void *f0 = nullptr, *f1 = nullptr;
		cudaDriverEntryPointQueryResult q0, q1;
		if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f0, 12000, cudaEnableDefault, &q0) != cudaSuccess ||
		    q0 != cudaDriverEntryPointSuccess || !f0 ||
		    cudaGetDriverEntryPointByVersion("cuCtxGetId", &f1, 12000, cudaEnableDefault, &q1) != cudaSuccess ||
		    q1 != cudaDriverEntryPointSuccess || !f1)
		{
			fprintf(stderr, "pgs: cuCtxGetCurrent / cuCtxGetId entry points unavailable\n");
			return PGS_ERROR_CUDA;
		}
		get_current = reinterpret_cast<CtxGetCurrent>(f0);
		get_id = reinterpret_cast<CtxGetId>(f1);
	}
	void *ctx = nullptr;
	unsigned long long id = 0;
	if (get_current(&ctx) != 0)
		return PGS_ERROR_NO_DEVICE;
	// No context current on this thread yet: cudaSetDevice binds (and, from
	// CUDA 12 on, initialises) the device's primary context.
	if (!ctx && (cudaSetDevice(dev) != cudaSuccess || get_current(&ctx) != 0))
		return PGS_ERROR_NO_DEVICE;
	if (!ctx || get_id(ctx, &id) != 0)
		return PGS_ERROR_NO_DEVICE;
	for (int i = 0; i < g_noalloc_num_slots; i++)
		if (g_noalloc_slots[i].ctx_id == id)
		{
			*out = g_noalloc_slots[i].ptr;
			return PGS_OK;
		}
	void *p = nullptr;
	cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_copy_scratch);
	if (e != cudaSuccess || !p)
	{
		fprintf(stderr, "pgs: cudaGetSymbolAddress(g_noalloc_copy_scratch) failed: %s\n", cudaGetErrorString(e));
		return PGS_ERROR_CUDA;
	}
	// Contexts that no longer exist keep their slots; past the table's size
	// the oldest slot is reused.
	int slot = g_noalloc_num_slots < NOALLOC_MAX_CONTEXTS ? g_noalloc_num_slots++ : int(id % NOALLOC_MAX_CONTEXTS);
	g_noalloc_slots[slot] = { id, static_cast<uint32_t *>(p) };
	*out = g_noalloc_slots[slot].ptr;
	return PGS_OK;
}
} // namespace

extern "C" {
void *pgs_cuda_backend_create(const pgs_cuda_backend_options *options, const pgs_backend_ops **ops, int *status)
{
	int dummy;
	if (!status)
		status = &dummy;
	auto *b = new (std::nothrow) CudaBackend();
	if (!b)
	{
		*status = PGS_ERROR_OUT_OF_MEMORY;
		return nullptr;
	}
	int r = b->init(options);
	if (r)
	{
		b->destroy();
		delete b;
		*status = r;
		return nullptr;
	}
	if (ops)
		*ops = &CUDA_OPS;
	*status = PGS_OK;
	return b;
}

int pgs_cuda_backend_begin_record(void *backend) { return backend ? B(backend)->begin_record() : PGS_ERROR_INVALID_ARGUMENT; }
int pgs_cuda_backend_end_record(void *backend) { return backend ? B(backend)->end_record() : PGS_ERROR_INVALID_ARGUMENT; }
int pgs_cuda_backend_replay(void *backend, uint32_t count, int reset_vram, int use_graph)
{
	return backend ? B(backend)->replay(count, reset_vram != 0, use_graph != 0) : PGS_ERROR_INVALID_ARGUMENT;
}
void *pgs_cuda_backend_stream(void *backend) { return backend ? static_cast<void *>(B(backend)->stream) : nullptr; }
int pgs_cuda_backend_sample_circuit(void *backend, const pgs_circuit_params *params, void *d_dst)
{
	if (!backend || !params || !d_dst)
		return PGS_ERROR_INVALID_ARGUMENT;
	return B(backend)->sample_circuit_device(*params, static_cast<uint32_t *>(d_dst));
}

// ---------------------------------------------------------------------------
// Batched replay.
struct pgs_batch
{
	BatchEngine e;
};

pgs_batch *pgs_batch_create(int device, int *status)
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
	auto *b = new (std::nothrow) pgs_batch();
	if (!b)
	{
		*status = PGS_ERROR_OUT_OF_MEMORY;
		return nullptr;
	}
	int r = b->e.init(device);
	if (r)
	{
		b->e.destroy();
		delete b;
		*status = r;
		return nullptr;
	}
	*status = PGS_OK;
	return b;
}

void pgs_batch_destroy(pgs_batch *batch)
{
	if (!batch)
		return;
	batch->e.destroy();
	delete batch;
}

int pgs_batch_add(pgs_batch *batch, void *cuda_backend)
{
	return batch && cuda_backend ? batch->e.add(B(cuda_backend)) : PGS_ERROR_INVALID_ARGUMENT;
}

int pgs_batch_replay(pgs_batch *batch, uint32_t count, int reset_vram, int use_graph)
{
	return batch ? batch->e.replay(count, reset_vram != 0, use_graph != 0) : PGS_ERROR_INVALID_ARGUMENT;
}

int pgs_batch_set_tuning(pgs_batch *batch, const pgs_batch_tuning *tuning)
{
	if (!batch || !tuning)
		return PGS_ERROR_INVALID_ARGUMENT;
	uint32_t block = tuning->cta_threads;
	if ((block != 128 && block != 256 && block != 512) || tuning->ctas_per_sm == 0 ||
	    tuning->ctas_per_sm * block > 1024)
		return PGS_ERROR_INVALID_ARGUMENT;
	batch->e.block = block;
	batch->e.ctas_per_sm = tuning->ctas_per_sm;
	batch->e.largest_first = tuning->largest_first != 0;
	batch->e.solo_min_prims = tuning->solo_min_prims;
	batch->e.invalidate();
	return PGS_OK;
}

int pgs_batch_get_tuning(pgs_batch *batch, pgs_batch_tuning *tuning)
{
	if (!batch || !tuning)
		return PGS_ERROR_INVALID_ARGUMENT;
	tuning->cta_threads = batch->e.block;
	tuning->ctas_per_sm = batch->e.ctas_per_sm;
	tuning->largest_first = batch->e.largest_first;
	tuning->solo_min_prims = batch->e.solo_min_prims;
	return PGS_OK;
}

int pgs_batch_autotune(pgs_batch *batch, uint32_t trials, int reset_vram, pgs_batch_tuning *best, float *best_ms)
{
	if (!batch || trials == 0)
		return PGS_ERROR_INVALID_ARGUMENT;
	BatchEngine &e = batch->e;
	static const pgs_batch_tuning candidates[] = {
		{ 128, 8, 1, 0 }, { 128, 4, 1, 0 }, { 256, 4, 1, 0 }, { 256, 2, 1, 0 }, { 512, 2, 1, 0 }, { 512, 1, 1, 0 },
		{ 256, 4, 0, 0 }, { 512, 2, 1, 100000 }, { 512, 2, 1, 50000 }, { 512, 2, 1, 20000 }, { 512, 2, 1, 10000 },
		{ 512, 2, 1, 5000 }, { 512, 2, 1, 2000 }, { 256, 4, 1, 20000 }, { 256, 4, 1, 5000 }, { 512, 2, 1, 1 },
	};
	cudaEvent_t ev[2];
	CUDA_TRY(cudaSetDevice(e.device));
	CUDA_TRY(cudaEventCreate(&ev[0]));
	CUDA_TRY(cudaEventCreate(&ev[1]));
	pgs_batch_tuning chosen = candidates[0];
	float chosen_ms = 0.0f;
	int r = PGS_OK;
	for (const pgs_batch_tuning &c : candidates)
	{
		r = pgs_batch_set_tuning(batch, &c);
		if (!r)
			r = e.replay(1, reset_vram != 0, true);  // builds the graph
		if (r)
			break;
		cudaEventRecord(ev[0], e.master);
		r = e.replay(trials, reset_vram != 0, true);
		cudaEventRecord(ev[1], e.master);
		if (r)
			break;
		float ms = 0.0f;
		if (cudaEventSynchronize(ev[1]) != cudaSuccess || cudaEventElapsedTime(&ms, ev[0], ev[1]) != cudaSuccess)
		{
			r = PGS_ERROR_CUDA;
			break;
		}
		ms /= float(trials);
		if (chosen_ms == 0.0f || ms < chosen_ms)
		{
			chosen = c;
			chosen_ms = ms;
		}
	}
	cudaEventDestroy(ev[0]);
	cudaEventDestroy(ev[1]);
	if (r)
		return r;
	r = pgs_batch_set_tuning(batch, &chosen);
	if (best)
		*best = chosen;
	if (best_ms)
		*best_ms = chosen_ms;
	return r;
}

void *pgs_batch_stream(pgs_batch *batch) { return batch ? static_cast<void *>(batch->e.master) : nullptr; }
uint32_t pgs_batch_launches_per_replay(pgs_batch *batch) { return batch ? batch->e.launches_per_replay : 0; }
int pgs_batch_synchronize(pgs_batch *batch)
{
	if (!batch)
		return PGS_ERROR_INVALID_ARGUMENT;
	CUDA_TRY(cudaSetDevice(batch->e.device));
	CUDA_TRY(cudaStreamSynchronize(batch->e.master));
	for (CudaBackend *b : batch->e.streams)
		CUDA_TRY(cudaStreamSynchronize(b->stream));
	return PGS_OK;
}
uint32_t pgs_cuda_backend_launches_per_replay(void *backend) { return backend ? B(backend)->launches_per_replay : 0; }
int pgs_cuda_backend_last_shade_ms(void *backend, float *ms)
{
	if (!backend || !ms)
		return PGS_ERROR_INVALID_ARGUMENT;
	CudaBackend *b = B(backend);
	if (!b->shade_timing)
		return PGS_ERROR_INVALID_ARGUMENT;
	if (cudaEventSynchronize(b->shade_ev[1]) != cudaSuccess)
		return PGS_ERROR_CUDA;
	if (cudaEventElapsedTime(ms, b->shade_ev[0], b->shade_ev[1]) != cudaSuccess)
		return PGS_ERROR_CUDA;
	return PGS_OK;
}

int pgs_cuda_backend_get_stats(void *backend, pgs_backend_stats *stats)
{
	if (!backend || !stats)
		return PGS_ERROR_INVALID_ARGUMENT;
	CudaBackend *b = B(backend);
	stats->h2d_bytes = b->h2d_bytes;
	stats->d2h_bytes = b->d2h_bytes;
	stats->kernel_launches = b->total_launches + b->launch_counter;
	stats->render_passes = b->render_passes;
	return PGS_OK;
}

int pgs_cuda_backend_set_shade_timing(void *backend, int enable)
{
	if (!backend)
		return PGS_ERROR_INVALID_ARGUMENT;
	CudaBackend *b = B(backend);
	b->shade_timing = enable != 0;
	if (b->graph_exec)
	{
		cudaGraphExecDestroy(b->graph_exec);
		b->graph_exec = nullptr;
	}
	return PGS_OK;
}
int pgs_cuda_backend_fragment_count(void *backend, uint64_t *count)
{
	if (!backend || !count)
		return PGS_ERROR_INVALID_ARGUMENT;
	unsigned long long v = 0;
	if (cudaMemcpy(&v, B(backend)->d_frags, sizeof(v), cudaMemcpyDeviceToHost) != cudaSuccess)
		return PGS_ERROR_CUDA;
	*count = v;
	return PGS_OK;
}
}

extern "C" int pgs_vram_local_copy_noalloc(void *vram, uint32_t num_planes, const pgs_copy_desc *desc, void *stream)
{
	if (!vram || !desc || num_planes == 0)
		return PGS_ERROR_INVALID_ARGUMENT;
	CopyParams c = {};
	uint64_t bb = desc->bitbltbuf;
	c.sbp = field(bb, 0, 14); c.sbw = field(bb, 16, 6); c.spsm = field(bb, 24, 6);
	c.dbp = field(bb, 32, 14); c.dbw = field(bb, 48, 6); c.dpsm = field(bb, 56, 6);
	c.ssax = field(desc->trxpos, 0, 11); c.ssay = field(desc->trxpos, 16, 11);
	c.dsax = field(desc->trxpos, 32, 11); c.dsay = field(desc->trxpos, 48, 11);
	c.width = field(desc->trxreg, 0, 12); c.height = field(desc->trxreg, 32, 12);
	c.xdir = field(desc->trxdir, 0, 2);
	c.invalidate_ss = num_planes > 1;
	if (c.xdir != LOCAL_TO_LOCAL)
		return PGS_ERROR_INVALID_ARGUMENT;
	if (c.width == 0 || c.height == 0)
		return PGS_OK;
	if (uint64_t(c.width) * c.height > PGS_NOALLOC_COPY_MAX_PIXELS)
	{
		fprintf(stderr, "pgs: pgs_vram_local_copy_noalloc: %ux%u pixels exceed the %u-pixel staging array\n",
		        c.width, c.height, PGS_NOALLOC_COPY_MAX_PIXELS);
		return PGS_ERROR_CAPACITY;
	}
	uint32_t *staging = nullptr;
	int r = noalloc_scratch(&staging);
	if (r)
		return r;
	cudaStream_t s = static_cast<cudaStream_t>(stream);
	dim3 grid((c.width + 31) / 32, (c.height + 7) / 8);
	noalloc_gather_kernel<<<grid, 256, 0, s>>>(c, static_cast<const uint8_t *>(vram), staging);
	noalloc_scatter_kernel<<<grid, 256, 0, s>>>(c, static_cast<uint8_t *>(vram), staging);
	cudaError_t e = cudaGetLastError();
	if (e != cudaSuccess)
	{
		fprintf(stderr, "pgs: pgs_vram_local_copy_noalloc launch failed: %s\n", cudaGetErrorString(e));
		return PGS_ERROR_CUDA;
	}
	return PGS_OK;
}
