/*
 * pgs.h -- C ABI of the GB300 Graphics Synthesizer backend.
 *
 * Two surfaces live here:
 *
 *  1. The frontend (pgs_gs_*): the reference's GSInterface public API
 *     (gs/gs_interface.hpp:251-304) re-hosted without Vulkan types.  It ingests
 *     GIF packets and A+D register writes, batches primitives into render
 *     passes, tracks page hazards and drives a backend.
 *
 *  2. The backend (pgs_backend_ops): the methods of the reference's GSRenderer
 *     that the frontend calls (gs/gs_renderer.hpp:244-323), as a table of plain
 *     C function pointers.  The CUDA backend (pgs_cuda_backend_*) implements it
 *     with hand-written sm_103a kernels.  Any other implementation of the table
 *     (for example a CPU checker) can be plugged under the same frontend.
 *
 * Record layouts (pgs_vertex_position, pgs_vertex_attribute,
 * pgs_primitive_attribute, pgs_state_vector) are bit-compatible with the
 * reference's shared CPU/GPU structures (gs/shaders/data_structures.h:55-80,
 * 139-144) so that a frontend written against the reference emits the same
 * bytes.  All entry points return 0 on success and a negative pgs_status on
 * failure unless documented otherwise; nothing here traps the GPU.
 */
#ifndef PGS_H_
#define PGS_H_

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define PGS_ABI_VERSION 6u
/* VRAM snapshots a render pass can hold (pgs_render_pass.snapshot_textures). */
#define PGS_MAX_VRAM_SNAPSHOTS 4u

/* ------------------------------------------------------------------ */
/* Status codes                                                        */
/* ------------------------------------------------------------------ */
typedef enum pgs_status
{
	PGS_OK = 0,
	PGS_ERROR_INVALID_ARGUMENT = -1,
	PGS_ERROR_OUT_OF_MEMORY = -2,
	PGS_ERROR_CUDA = -3,
	PGS_ERROR_NO_DEVICE = -4,
	PGS_ERROR_UNSUPPORTED = -5,
	/* Sticky device-side error: a capacity limit was hit or a bounded wait
	 * expired.  Query with pgs_backend_ops.get_error. */
	PGS_ERROR_DEVICE_FLAG = -6,
	PGS_ERROR_CAPACITY = -7,
	/* A file could not be opened, read or written, or is not a GS dump. */
	PGS_ERROR_IO = -8
} pgs_status;

/* ------------------------------------------------------------------ */
/* Limits (gs/gs_renderer.hpp:154-160, gs/shaders/data_structures.h)   */
/* ------------------------------------------------------------------ */
#define PGS_VRAM_SIZE (4u * 1024u * 1024u)
#define PGS_MAX_PRIMITIVES_PER_FLUSH (64u * 1024u)
#define PGS_MAX_RENDER_PASS_INSTANCES 8u
#define PGS_MAX_TEXTURES 4096u
#define PGS_MAX_STATE_VECTORS 4096u
#define PGS_CLUT_INSTANCES 1024u
#define PGS_CLUT_SIZE_BYTES 1024u

/* ------------------------------------------------------------------ */
/* Primitive records written by the frontend                            */
/* ------------------------------------------------------------------ */

/* VertexPosition (gs/shaders/data_structures.h:55-58): 12.4 fixed-point
 * window coordinates after XYOFFSET, 32-bit Z. */
typedef struct pgs_vertex_position
{
	int32_t x, y;
	uint32_t z;
	int32_t padding;
} pgs_vertex_position;

/* VertexAttribute (gs/shaders/data_structures.h:61-68). */
typedef struct pgs_vertex_attribute
{
	float s, t, q;
	uint32_t rgba;
	float fog;
	uint16_t u, v;
} pgs_vertex_attribute;

/* PrimitiveAttribute (gs/shaders/data_structures.h:71-80).  bb is the
 * scissored pixel bounding box (lo.x, lo.y, hi.x, hi.y), inclusive. */
typedef struct pgs_primitive_attribute
{
	int16_t bb[4];
	uint32_t state;
	uint32_t tex;
	uint32_t tex2;
	uint32_t alpha;
	uint32_t fbmsk;
	uint32_t fogcol;
} pgs_primitive_attribute;

/* StateVector (gs/shaders/data_structures.h:139-144). */
typedef struct pgs_state_vector
{
	uint32_t combiner;
	uint32_t blend_mode;
	uint32_t dimx_lo, dimx_hi;
} pgs_state_vector;

/* Texture descriptor.  The reference samples an RGBA8 image decoded by
 * upload.comp (TexInfo, gs/shaders/data_structures.h:98-105, built at
 * gs/gs_interface.cpp:1752-1790).  This backend samples swizzled VRAM and the
 * CLUT directly, so the descriptor carries the raw addressing state instead. */
typedef struct pgs_texture_desc
{
	uint32_t tbp0;          /* TEX0.TBP0, 256-byte blocks */
	uint32_t tbw;           /* TEX0.TBW, 64-pixel units */
	uint32_t psm;           /* TEX0.PSM */
	uint32_t tw_log2, th_log2;
	uint32_t cpsm;          /* CLUT format (PSMCT32 or PSMCT16/16S) */
	uint32_t csa;           /* CLUT offset in 16-entry banks */
	uint32_t clut_instance; /* CLUT ring slot holding the palette */
	uint32_t aem, ta0, ta1; /* TEXA */
	uint32_t wms, wmt;      /* CLAMP wrap modes */
	uint32_t minu, maxu, minv, maxv;
	/* Mip levels sampled (1..7; 1 unless TEX1.MMIN selects a mipmap mode):
	 * min(MXL + 1, min(TW, TH) + 1, 7) as compute_effective_texture_rect
	 * (gs/gs_renderer.cpp:1235-1265).  mip[l - 1] = TBP | TBW << 16 of level l
	 * from MIPTBP1 / MIPTBP2; zero for levels not sampled. */
	uint32_t levels;
	uint32_t mip[6];
	/* Super-sampled texture (levels == 1): 1 + the frame's samples per pixel
	 * layers -- layer 0 the single-sampled image, layer s + 1 sample s read
	 * through the reference plane (create_cached_texture with desc.samples,
	 * gs/gs_renderer.cpp:1317-1386; upload.comp SUPER_SAMPLED).  0 or 1: a
	 * plain texture. */
	uint32_t samples;
	/* TEX1.MXL as written (0 without a mipmapping MMIN).  Backends ignore it;
	 * it keeps textures that differ only in it apart, as the reference's
	 * texture key does (gs/gs_interface.cpp:1605-1619). */
	uint32_t mxl;
} pgs_texture_desc;

/* One framebuffer instance inside a render pass (RenderPass::Instance,
 * gs/gs_renderer.hpp:174-227). */
typedef struct pgs_rp_instance
{
	uint64_t frame;          /* FRAME_n register bits */
	uint64_t zbuf;           /* ZBUF_n register bits */
	int32_t base_x, base_y;  /* pixel origin of the coarse tile grid */
	uint32_t coarse_tiles_width, coarse_tiles_height;
	uint32_t sampling_rate_x_log2, sampling_rate_y_log2;
	uint32_t opaque_fbmask;
	uint32_t z_sensitive, z_write, channel_shuffle;
} pgs_rp_instance;

/* Why a render pass ended (FlushReason, gs/page_tracker.hpp:117-126). */
typedef enum pgs_flush_reason
{
	PGS_FLUSH_FB_POINTER = 0,     /* frame/depth buffer change with no instance left */
	PGS_FLUSH_OVERFLOW = 1,       /* primitive, state, texture or CLUT table full */
	PGS_FLUSH_TEXTURE_HAZARD = 2, /* texture or CLUT read of pages the pass wrote */
	PGS_FLUSH_COPY_HAZARD = 3,    /* transfer touching pages the pass reads or writes */
	PGS_FLUSH_SUBMISSION = 4,     /* explicit flush, vsync, host access to VRAM */
	PGS_FLUSH_PRESSURE = 5,       /* pending-work limits reached */
	PGS_FLUSH_HOST_ACCESS = 6     /* LOCAL->HOST read-back of pages the pass wrote */
} pgs_flush_reason;

typedef struct pgs_render_pass
{
	const pgs_vertex_position *positions;     /* 3 per primitive */
	const pgs_vertex_attribute *attributes;   /* 3 per primitive */
	const pgs_primitive_attribute *prims;
	uint32_t num_primitives;

	const pgs_state_vector *states;
	uint32_t num_states;
	const pgs_texture_desc *textures;
	uint32_t num_textures;

	pgs_rp_instance instances[PGS_MAX_RENDER_PASS_INSTANCES];
	uint32_t num_instances;
	uint32_t coarse_tile_size_log2;
	uint32_t has_aa1, has_scanmsk;
	uint32_t flush_reason;  /* pgs_flush_reason */
	/* Some primitive samples mip levels (TEX1.MXL > 0 with a mipmapping MMIN). */
	uint32_t has_mipmap;
	/* Some texture of the pass is super-sampled (pgs_texture_desc.samples). */
	uint32_t has_ss_textures;
	/* Field-aware rendering (GSRenderer::set_field_aware_super_sampling,
	 * gs/gs_renderer.cpp:355-358): instances that end at or above row 256
	 * shade every covered tile super-sampled with rows snapped at half the
	 * sample pitch, and blur kernels keep per-sample textures.  ABI >= 4. */
	uint32_t field_aware;
	/* Hacks::allow_blend_demote (gs/gs_interface.hpp:231-236): when every
	 * state blends, coarse tiles with 32 or more primitives and no depth
	 * write shade single-sampled.  ABI >= 4. */
	uint32_t blend_demote;
	/* ABI >= 5.  VRAM snapshots the frontend took during the pass
	 * (pgs_backend_ops.snapshot_vram): textures [snapshot_textures[k - 1],
	 * snapshot_textures[k]) decode from snapshot k (the first from 0), the
	 * rest from VRAM as the pass begins.  The reference samples textures from
	 * cache images uploaded before a transfer can overwrite their source
	 * (flush_cache_upload via PageTracker::flush_cached,
	 * gs/page_tracker.cpp:585-594); this backend decodes a pass's textures
	 * when the pass begins, so a transfer into a texture the open pass holds
	 * is preceded by a snapshot instead. */
	uint32_t num_snapshots;
	uint32_t snapshot_textures[PGS_MAX_VRAM_SNAPSHOTS];
} pgs_render_pass;

/* A VRAM transfer (CopyDescriptor, gs/gs_renderer.hpp).  For HOST_TO_LOCAL,
 * host_data points at the HWREG payload received so far; bytes below
 * host_offset were already written by an earlier partial flush. */
typedef struct pgs_copy_desc
{
	uint64_t bitbltbuf, trxpos, trxreg, trxdir;
	const void *host_data;
	uint64_t host_size;      /* bytes available in host_data */
	uint64_t host_offset;    /* bytes already consumed */
	uint64_t host_required;  /* bytes of the whole transfer */
} pgs_copy_desc;

/* A CLUT load (PaletteUploadDescriptor, gs/gs_renderer.hpp). */
typedef struct pgs_palette_upload
{
	uint64_t tex0;       /* TEX0 with CPSM/CSA/CSM/CBP normalised */
	uint64_t texclut;
	float csm2_x_scale;
	uint32_t csm2_x_bias;
	uint32_t base_instance;  /* CLUT state the load starts from */
	/* ABI >= 5: 1 + the CLUT ring slot the load writes.  The frontend numbers
	 * the ring as the reference's renderer does (update_palette_cache,
	 * rewind_clut_instance, gs/gs_renderer.cpp:3384-3419): a load that nothing
	 * has read yet is rewritten in place by a load replacing it, and a pass
	 * that ends on an older memoised palette rewinds the ring to it.  0: the
	 * backend takes the slot after the last one it wrote. */
	uint32_t target;
} pgs_palette_upload;

/* FlushStats (gs/gs_renderer.hpp:55-65) plus fragment counters. */
typedef struct pgs_flush_stats
{
	uint64_t num_render_passes;
	uint64_t num_primitives;
	uint64_t num_copies;
	uint64_t num_palette_updates;
	uint64_t num_copy_barriers;
	uint64_t num_flushes_by_reason[8];
} pgs_flush_stats;

/* ------------------------------------------------------------------ */
/* Backend interface (replaces GSRenderer)                              */
/* ------------------------------------------------------------------ */
/* One CRTC circuit read-out (sample_circuit.frag, gs/shaders/sample_circuit.frag:98-148,
 * as set up by GSRenderer::sample_crtc_circuit, gs/gs_renderer.cpp:4055-4112).
 * The output is width x height RGBA8; texels outside valid_width x
 * valid_height are zero (the render pass clear). */
typedef struct pgs_circuit_params
{
	uint32_t fbp, fbw, psm, dbx, dby;   /* DISPFB fields */
	uint32_t phase, phase_stride;       /* first line offset and line step */
	uint32_t super_samples;             /* 1, or 4 / 8 / 16 for a 2x2 high-resolution read-out */
	uint32_t width, height;             /* output image extent */
	uint32_t valid_width, valid_height; /* sampled part (scissor) */
} pgs_circuit_params;

/* Output merge of one vsync (GSRenderer::vsync, gs/gs_renderer.cpp:4189-5055),
 * computed by the frontend from the privileged registers; a backend samples the
 * circuits, composes them, performs the EXTWRITE write-back into VRAM and
 * deinterlaces. */
typedef struct pgs_merge_params
{
	pgs_circuit_params circuit[2]; /* read-out of each circuit; width == 0: not sampled */
	int32_t rect_x[2], rect_y[2];  /* viewport of each circuit in the merged image */
	uint32_t rect_w[2], rect_h[2]; /* 0 x 0: circuit not drawn */
	uint32_t width, height;        /* merged image */
	uint32_t draw_circuit2;        /* SLBG = 0: circuit 2 is drawn first, unblended */
	uint32_t draw_circuit1;
	uint32_t blend;                /* circuit 1 over circuit 2 / background: 0 replace,
	                                * 1 constant ALP, 2 circuit 1 alpha (PMODE.MMOD) */
	uint32_t alp;
	uint32_t bgcolor;              /* background RGB (BGCOLOR); background alpha is 0 */
	/* EXTWRITE feedback write (extwrite.comp:37-98). */
	uint32_t ext_write;
	uint32_t ext_source;           /* 0 merged image, 1 circuit 2, 2 circuit 1 */
	uint32_t ext_width, ext_height;
	uint32_t ext_wdx, ext_wdy, ext_exbp, ext_exbw, ext_emoda, ext_emodc;
	float ext_uv_base[2], ext_uv_scale[2];
	/* FastMAD deinterlace over the last four merged fields (weave.frag). */
	uint32_t deinterlace;          /* 0: output the merged image, drop the field history */
	uint32_t phase;
	uint32_t raw_circuit;          /* 1 / 2: output that circuit's read-out as it is */
	uint32_t padding;
} pgs_merge_params;

typedef struct pgs_backend_ops
{
	uint32_t abi_version;
	void (*destroy)(void *self);
	/* GSRenderer::reserve_primitive_buffers + get_reserved_* (gs/gs_renderer.hpp:251-254).
	 * The frontend writes records straight into backend-owned host memory; the
	 * buffers belong to the backend again from flush_rendering until the next
	 * reserve_primitive_buffers call. */
	int (*reserve_primitive_buffers)(void *self, uint32_t num_primitives,
	                                 pgs_vertex_position **positions,
	                                 pgs_vertex_attribute **attributes,
	                                 pgs_primitive_attribute **prims);
	/* GSRenderer::flush_rendering(const RenderPass &) (gs/gs_renderer.cpp:3126-3285). */
	int (*flush_rendering)(void *self, const pgs_render_pass *rp);
	/* GSRenderer::copy_vram (gs/gs_renderer.cpp:2829-2867). */
	int (*copy_vram)(void *self, const pgs_copy_desc *desc);
	/* GSRenderer::update_palette_cache (gs/gs_renderer.cpp:3400-3419).  Returns the
	 * new CLUT instance (>= 0) or a negative pgs_status. */
	int (*update_palette_cache)(void *self, const pgs_palette_upload *upload);
	/* GSRenderer::invalidate_super_sampling_state (gs/gs_renderer.cpp:316-341). */
	int (*set_super_sampling)(void *self, uint32_t rate_x_log2, uint32_t rate_y_log2);
	/* GSRenderer::flush_submit (gs/gs_renderer.cpp:1091-1187). */
	int (*flush_submit)(void *self);
	/* flush_readback + map_vram_read: blocks until all submitted work is done,
	 * then copies [offset, offset+size) of VRAM plane `plane` into dst.
	 * Plane 0 is the single-sampled GS VRAM, plane 1 the super-sample
	 * reference plane, planes 2.. the samples. */
	int (*read_vram)(void *self, uint32_t plane, uint64_t offset, uint64_t size, void *dst);
	/* map_vram_write/end_vram_write: host writes into plane 0. */
	int (*write_vram)(void *self, uint64_t offset, uint64_t size, const void *src);
	/* Sticky device error flags (bin overflow, bounded-wait expiry). */
	int (*get_error)(void *self, uint32_t *flags);
	/* abi_version >= 2, optional (NULL: the frontend reads synchronously).
	 * Queues a copy of [offset, offset+size) of plane 0 into dst behind all
	 * submitted work and returns a ticket; dst must stay valid and untouched
	 * until wait_ticket(ticket) returns.  This is the asynchronous side of the
	 * reference's timeline-semaphore readback (GSRenderer::flush_readback +
	 * wait_timeline, gs/gs_renderer.cpp:1037). */
	int (*read_vram_async)(void *self, uint64_t offset, uint64_t size, void *dst, uint64_t *ticket);
	int (*wait_ticket)(void *self, uint64_t ticket);
	/* abi_version >= 2, optional: CRTC circuit read-out of the current VRAM into
	 * host memory dst (params->width * params->height * 4 bytes). */
	int (*sample_circuit)(void *self, const pgs_circuit_params *params, void *dst);
	/* abi_version >= 3, optional: one vsync's output into host memory dst
	 * (raw circuit: its read-out; deinterlaced: width x 2 * height; else
	 * width x height RGBA8). */
	int (*vsync)(void *self, const pgs_merge_params *params, void *dst);
	/* abi_version >= 4, optional: GPU time per stage (GSRenderer timestamps,
	 * gs/gs_renderer.cpp:1205-1233).  enable 1 starts timing the stages, 0
	 * stops it, -1 leaves it as it is; totals (PGS_TIMESTAMP_COUNT doubles,
	 * may be NULL) receives the seconds accumulated so far per stage, after
	 * the timed work has completed. */
	int (*timestamps)(void *self, int enable, double *totals);
	/* abi_version >= 5, optional (NULL: the frontend ends the pass instead).
	 * Copies every VRAM plane, behind all submitted work, into the next of
	 * the PGS_MAX_VRAM_SNAPSHOTS snapshot slots of the open render pass and
	 * returns the slot (>= 0) or a negative pgs_status.  flush_rendering
	 * decodes the pass's textures from the snapshots pgs_render_pass names and
	 * releases the slots. */
	int (*snapshot_vram)(void *self);
	/* abi_version >= 6, optional (NULL: the frontend reads plane 0 whole and
	 * de-swizzles it on the host).  LOCAL->HOST read-out of the source
	 * rectangle desc names (BITBLTBUF SBP/SBW/SPSM, TRXPOS SSAX/SSAY, TRXREG),
	 * as vram_readback packs it (gs/gs_util.hpp:50-110): pixels in row order,
	 * 4, 3, 2 or 1 bytes each for the 32-, 24-, 16- and 8-bit formats, the
	 * 4-bit formats unsupported (nothing written).  Reads plane 0 behind all
	 * submitted work and returns when dst (dst_size bytes, at least the
	 * rectangle's) holds the result. */
	int (*readback_rect)(void *self, const pgs_copy_desc *desc, void *dst, uint64_t dst_size);
} pgs_backend_ops;

/* TimestampType (gs/gs_renderer.hpp:67-79). */
#define PGS_TIMESTAMP_SYNC_HOST_TO_VRAM 0u
#define PGS_TIMESTAMP_COPY_VRAM 1u
#define PGS_TIMESTAMP_PALETTE_UPDATE 2u
#define PGS_TIMESTAMP_TEXTURE_UPLOAD 3u
#define PGS_TIMESTAMP_TRIANGLE_SETUP 4u
#define PGS_TIMESTAMP_BINNING 5u
#define PGS_TIMESTAMP_SHADING 6u
#define PGS_TIMESTAMP_READBACK 7u
#define PGS_TIMESTAMP_VSYNC 8u
#define PGS_TIMESTAMP_COUNT 9u

/* ------------------------------------------------------------------ */
/* CUDA backend                                                         */
/* ------------------------------------------------------------------ */
typedef struct pgs_cuda_backend_options
{
	int device;                  /* CUDA ordinal */
	uint32_t max_samples_log2;   /* 0..4: VRAM holds 2 + 2^max planes */
	uint32_t flags;
	uint32_t arena_mib;          /* initial record arena (MiB); 0 = 256.  It grows on demand. */
} pgs_cuda_backend_options;

/* Creates a backend on `device`; returns NULL and sets *status on failure
 * (PGS_ERROR_NO_DEVICE when no GPU is visible).  *ops receives the table. */
void *pgs_cuda_backend_create(const pgs_cuda_backend_options *options,
                              const pgs_backend_ops **ops, int *status);

/* Frame programs: the backend records every op between begin and end into
 * device-resident form, so the same frame can be replayed with no host
 * traffic (and captured into a CUDA graph). */
int pgs_cuda_backend_begin_record(void *backend);
int pgs_cuda_backend_end_record(void *backend);
/* Replays the recorded program `count` times on the backend's stream.  When
 * reset_vram is non-zero every replay starts from the VRAM image that was
 * current at begin_record. */
int pgs_cuda_backend_replay(void *backend, uint32_t count, int reset_vram, int use_graph);
/* Returns the cudaStream_t the backend launches on, as an opaque pointer. */
void *pgs_cuda_backend_stream(void *backend);
/* Kernel launches issued by the last replay (per replay). */
uint32_t pgs_cuda_backend_launches_per_replay(void *backend);
/* Device time from the first to the last shading kernel of the last replay,
 * in milliseconds (CUDA events on the backend's stream). */
int pgs_cuda_backend_last_shade_ms(void *backend, float *ms);
/* Covered pixel samples (primitive x sample pairs that passed the coverage
 * test) counted by the shading kernels since the backend was created. */
int pgs_cuda_backend_fragment_count(void *backend, uint64_t *count);

typedef struct pgs_backend_stats
{
	uint64_t h2d_bytes;     /* host->device bytes copied since creation */
	uint64_t d2h_bytes;     /* device->host bytes copied since creation */
	uint64_t kernel_launches;
	uint64_t render_passes;
} pgs_backend_stats;

/* CRTC circuit read-out (pgs_circuit_params) of the backend's VRAM into device
 * memory d_dst (width * height * 4 bytes), queued on the backend's stream. */
int pgs_cuda_backend_sample_circuit(void *backend, const pgs_circuit_params *params, void *d_dst);

/* Transfer and launch counters of the backend. */
int pgs_cuda_backend_get_stats(void *backend, pgs_backend_stats *stats);
/* When enabled, every replay records CUDA events (also inside the replay's
 * CUDA graph) around the shading kernels of its render passes; the time
 * between them is returned by pgs_cuda_backend_last_shade_ms once the replay
 * has completed. */
int pgs_cuda_backend_set_shade_timing(void *backend, int enable);

/* ------------------------------------------------------------------ */
/* Batched replay of many command streams                               */
/* ------------------------------------------------------------------ */
/* Many independent GS command streams, each recorded into its own CUDA
 * backend (pgs_cuda_backend_begin_record / end_record), replayed together:
 * every round takes each stream one render pass further, and one persistent
 * kernel launch shades the current pass of all streams; the schedule is a
 * single CUDA graph.  No counterpart in the reference, which renders one
 * stream per GSInterface. */
typedef struct pgs_batch pgs_batch;

typedef struct pgs_batch_tuning
{
	uint32_t cta_threads;    /* 128, 256 or 512 */
	uint32_t ctas_per_sm;    /* persistent CTAs per SM (1 .. 1024 / cta_threads) */
	uint32_t largest_first;  /* order work items by size within a round */
	/* Streams with at least this many primitives per frame run as their own
	 * branch of the replay graph (their passes back to back on their own
	 * stream, no round barriers); the others share the batched kernel.
	 * 0: every stream goes through the rounds. */
	uint32_t solo_min_prims;
} pgs_batch_tuning;

pgs_batch *pgs_batch_create(int device, int *status);
void pgs_batch_destroy(pgs_batch *batch);
/* Adds a CUDA backend that holds a recorded frame; the backend must outlive
 * the batch and not be replayed on its own while the batch is in use. */
int pgs_batch_add(pgs_batch *batch, void *cuda_backend);
/* Replays every stream `count` times (from its begin_record VRAM when
 * reset_vram is set), as a CUDA graph when use_graph is set. */
int pgs_batch_replay(pgs_batch *batch, uint32_t count, int reset_vram, int use_graph);
int pgs_batch_set_tuning(pgs_batch *batch, const pgs_batch_tuning *tuning);
int pgs_batch_get_tuning(pgs_batch *batch, pgs_batch_tuning *tuning);
/* Times `trials` graph replays of each candidate tuning (CTA size x CTAs per
 * SM x item order) and keeps the fastest; *best receives it, *best_ms its
 * mean time per replay. */
int pgs_batch_autotune(pgs_batch *batch, uint32_t trials, int reset_vram, pgs_batch_tuning *best, float *best_ms);
/* The batch's cudaStream_t (graph launches go there), as an opaque pointer. */
void *pgs_batch_stream(pgs_batch *batch);
/* Kernel launches of one batched replay. */
uint32_t pgs_batch_launches_per_replay(pgs_batch *batch);
/* Waits for every replay issued so far; afterwards each stream's VRAM can be
 * read through its backend. */
int pgs_batch_synchronize(pgs_batch *batch);

/* ------------------------------------------------------------------ */
/* Learned anti-aliasing upscaler                                       */
/* ------------------------------------------------------------------ */
/* A 6-layer 3x3 convolutional network (32 channels, ReLU, residual over the
 * input) that maps a 1x RGBA8 render to an estimate of the same scene's 16x
 * SSAA resolve, with BF16 tensor-core forward and backward kernels (FP32
 * accumulation) and an Adam step on FP32 master weights.  No counterpart in
 * the reference.  Images are n x h x w x 4 bytes in device memory.  Parameters
 * are a flat FP32 vector: per layer the weights [tap][out][in] then the biases;
 * layer shapes 4->32, 32->32 (x4), 32->4. */
void *pgs_upscaler_create(int device, int *status);
void pgs_upscaler_destroy(void *upscaler);
uint32_t pgs_upscaler_param_count(void *upscaler);
/* Sets the weights and resets the optimiser state. */
int pgs_upscaler_set_params(void *upscaler, const float *params, uint32_t count);
int pgs_upscaler_get_params(void *upscaler, float *params, uint32_t count);
/* Gradient of the last backward call (same layout as the parameters). */
int pgs_upscaler_get_gradient(void *upscaler, float *grad, uint32_t count);
/* Inference; d_out_rgba receives the clamped RGBA8 result. */
int pgs_upscaler_forward(void *upscaler, const void *d_images, uint32_t n, uint32_t h, uint32_t w, void *d_out_rgba);
/* Forward + mean-squared-error loss against d_targets + backward; *loss (may
 * be NULL) receives the loss and waits for it. */
int pgs_upscaler_backward(void *upscaler, const void *d_images, const void *d_targets, uint32_t n, uint32_t h,
                          uint32_t w, double *loss);
int pgs_upscaler_adam_step(void *upscaler, float learning_rate);
/* 32->32 layers on tcgen05 with TMA-fed operands and TMEM accumulators, with
 * 1 or 2 persistent CTAs per SM (2 is the default), or on the mma.sync path
 * (0). */
int pgs_upscaler_set_tensor_path(void *upscaler, int tcgen05);
/* Sticky error flags of the tcgen05 kernels (a bounded wait that ran out). */
int pgs_upscaler_get_error(void *upscaler, uint32_t *flags);
/* The stream the upscaler queues its work on (a cudaStream_t, as an opaque
 * pointer): its own stream unless pgs_upscaler_set_stream chose another. */
void *pgs_upscaler_stream(void *upscaler);
/* Queues the upscaler's later work on `stream` (a cudaStream_t of the same
 * device, e.g. a backend's stream, so that a frame's rendering and its
 * upscaling follow each other with no cross-stream wait); NULL selects the
 * upscaler's own stream again.  Waits for the work queued so far first.  The
 * caller keeps `stream` alive while it is selected. */
int pgs_upscaler_set_stream(void *upscaler, void *stream);
/* Self-test of the tcgen05 tensor-core path: a 128x32x32 BF16 product from
 * shared memory (mode 0: no-swizzle operand layout, 1: 64-byte swizzle) read
 * back from tensor memory into out (128 x 32 floats, row-major).  Mode 2
 * issues nothing and waits on the completion barrier with a short limit: the
 * wait runs out, the kernel releases its tensor memory and returns, and the
 * call reports PGS_ERROR_DEVICE_FLAG (the bounded-wait failure path). */
int pgs_umma_selftest(int device, uint32_t mode, float *out);
int pgs_upscaler_synchronize(void *upscaler);

/* ------------------------------------------------------------------ */
/* Allocation-free local->local VRAM copy                               */
/* ------------------------------------------------------------------ */
/* No counterpart in the reference.  For callers that cannot allocate device
 * memory — code running under a pool-restricted allocator, inside another
 * framework's arena, or with a hard no-cudaMalloc rule on a
 * latency-critical path — this performs the LOCAL_TO_LOCAL transfer described
 * by desc (BITBLTBUF/TRXPOS/TRXREG, XDIR = 2) on a caller-owned VRAM image
 * without allocating anything.  vram points to num_planes consecutive 4 MiB
 * planes in device memory (plane 1, when present, is the super-sample
 * reference plane whose written bits are cleared as by copy_vram); stream is
 * a cudaStream_t or NULL.  Results equal those of copy_vram: every source
 * pixel is read before any destination pixel is written.
 *
 * The source rectangle is staged in a fixed device array of
 * PGS_NOALLOC_COPY_MAX_PIXELS 32-bit entries (1 MiB) that every GPU loading the
 * library holds until exit; larger rectangles are rejected with
 * PGS_ERROR_CAPACITY.  The first call in a CUDA context looks up that array's
 * device address (cudaGetSymbolAddress) with the context current and keeps it
 * for that context; make that first call before any stream capture.  A context
 * that is destroyed and created again (cudaDeviceReset) counts as a new one, so
 * the lookup runs again there.  All calls share the array, so calls whose work
 * overlaps on the GPU race; serialise them on one stream.  Nothing in the array
 * needs to start at zero: each call overwrites the entries it reads. */
#define PGS_NOALLOC_COPY_MAX_PIXELS (256u * 1024u)
int pgs_vram_local_copy_noalloc(void *vram, uint32_t num_planes, const pgs_copy_desc *desc, void *stream);

/* ------------------------------------------------------------------ */
/* Frontend (GSInterface)                                               */
/* ------------------------------------------------------------------ */
typedef struct pgs_gs pgs_gs;

typedef struct pgs_gs_options
{
	/* sizeof(pgs_gs_options) as the caller was built; fields past it read as
	 * zero, so a caller built against a shorter layout keeps working.  0 means
	 * the whole current layout. */
	uint32_t struct_size;
	/* 1, 2, 4, 8 or 16 (SuperSampling enum).  Lowered to the most the backend
	 * was created for, as set_super_sampling_rate does with
	 * get_max_supported_super_sampling (gs/gs_interface.cpp:69-70). */
	uint32_t super_sampling;
	uint32_t ordered_super_sampling;
	uint32_t vram_size;           /* must be PGS_VRAM_SIZE */
	/* GSOptions::dynamic_super_sampling: accepted and not needed -- the rate
	 * can always change in flight, limited to the sample planes the backend
	 * was created with (pgs_cuda_backend_options.max_samples_log2). */
	uint32_t dynamic_super_sampling;
	/* GSOptions::super_sampled_textures (pgs_gs_set_super_sampled_textures);
	 * off when the resulting rate is 1x. */
	uint32_t super_sampled_textures;
	/* PGS_THREADED_DECODE_*: whether a GIF transfer is decoded on a worker
	 * thread of the interface while the calling thread runs the state side
	 * (hazard tracking, render passes, backend calls and host callbacks stay
	 * on the calling thread, in stream order).  The results are the same
	 * either way.  Not part of the reference's GSOptions. */
	uint32_t threaded_decode;
} pgs_gs_options;

/* Transfers of 256 KiB and more are decoded on the worker thread. */
#define PGS_THREADED_DECODE_AUTO 0u
/* Every transfer is decoded on the calling thread. */
#define PGS_THREADED_DECODE_OFF 1u
/* Every transfer is decoded on the worker thread. */
#define PGS_THREADED_DECODE_ALWAYS 2u

/* GSInterface::init.  The frontend does not own the backend. */
pgs_gs *pgs_gs_create(const pgs_backend_ops *ops, void *backend, const pgs_gs_options *options,
                      int *status);
void pgs_gs_destroy(pgs_gs *gs);
/* GSInterface::gif_transfer.  size must be a multiple of 16 bytes. */
int pgs_gs_gif_transfer(pgs_gs *gs, uint32_t path, const void *data, size_t size);
/* GSInterface::write_register (A+D address map, gs/gs_register_addr.hpp). */
int pgs_gs_write_register(pgs_gs *gs, uint32_t addr, uint64_t payload);
/* GSInterface::flush. */
int pgs_gs_flush(pgs_gs *gs);
/* GSInterface::map_vram_read: flushes, waits and copies plane 0. */
int pgs_gs_read_vram(pgs_gs *gs, uint64_t offset, uint64_t size, void *dst);
/* Flushes like pgs_gs_read_vram but only queues the copy: *ticket names it, and
 * dst holds the VRAM contents as of this call once pgs_gs_wait(ticket) has
 * returned.  Lets the caller decode the next frame while this one renders
 * (the reference's asynchronous timeline, GSInterface + GSRenderer::wait_timeline,
 * gs/gs_renderer.cpp:1037).  With a backend that has no asynchronous read the
 * copy is made before returning and the ticket is 0. */
int pgs_gs_read_vram_async(pgs_gs *gs, uint64_t offset, uint64_t size, void *dst, uint64_t *ticket);
int pgs_gs_wait(pgs_gs *gs, uint64_t ticket);

/* GS dumps (the PCSX2 / GSdx dump format read by GSDumpParser,
 * dump/gs_dump_parser.cpp:8-263, and written by GSDumpGenerator,
 * dump/gs_dump_generator.cpp:104-237): header, register file, 4 MiB VRAM,
 * GIF path state, internal Q and privileged registers, then packets (0 GIF
 * transfer, 1 vsync, 2 FIFO read, 3 privileged registers).
 *
 * pgs_gs_dump_open restores the dump's start state into gs; each
 * pgs_gs_dump_next_vsync call then replays packets up to the next vsync that
 * follows a transfer (*field = its field) and returns 1, or 0 at the end of
 * the dump. */
int pgs_gs_dump_open(pgs_gs *gs, const char *path);
int pgs_gs_dump_next_vsync(pgs_gs *gs, uint32_t *field);
int pgs_gs_dump_close(pgs_gs *gs);
/* Recording: writes the header and gs's current state to path; afterwards
 * every pgs_gs_gif_transfer and pgs_gs_write_register is appended as a
 * transfer packet until pgs_gs_dump_record_end.  pgs_gs_dump_record_vsync
 * appends the privileged registers and a vsync packet. */
int pgs_gs_dump_record_begin(pgs_gs *gs, const char *path);
int pgs_gs_dump_record_vsync(pgs_gs *gs, uint32_t field);
int pgs_gs_dump_record_end(pgs_gs *gs);

/* Privileged registers (GSInterface::get_priv_register_state, gs/gs_interface.hpp:70-108):
 * index 0 PMODE, 1 SMODE1, 2 SMODE2, 3 SRFSH, 4 SYNCH1, 5 SYNCH2, 6 SYNCV,
 * 7 DISPFB1, 8 DISPLAY1, 9 DISPFB2, 10 DISPLAY2, 11 EXTBUF, 12 EXTDATA,
 * 13 EXTWRITE, 14 BGCOLOR. */
int pgs_gs_write_priv_register(pgs_gs *gs, uint32_t index, uint64_t value);
int pgs_gs_read_priv_register(pgs_gs *gs, uint32_t index, uint64_t *value);

#define PGS_SCANOUT_FORCE_PROGRESSIVE 1u
#define PGS_SCANOUT_HIGH_RESOLUTION 2u
/* CRTC read-out of circuit 0 or 1 (DISPFB1/DISPLAY1 or DISPFB2/DISPLAY2) for
 * field `phase`, as GSRenderer::vsync samples it (compute_circuit_rect +
 * sample_crtc_circuit, gs/gs_renderer.cpp:4055-4172, 4547-4560): flushes, then
 * writes the RGBA8 circuit image into dst (capacity dst_size bytes) and its
 * extent into *width / *height.  With PGS_SCANOUT_HIGH_RESOLUTION and a
 * super-sampled frame scanned out progressively, the image is 2x2 larger and
 * resolves the sample planes.  Circuit merging, PMODE blending and CRTC
 * timings are not applied. */
int pgs_gs_scanout_circuit(pgs_gs *gs, uint32_t circuit, uint32_t phase, uint32_t flags, void *dst, uint64_t dst_size,
                           uint32_t *width, uint32_t *height);

/* vsync (GSInterface::vsync -> GSRenderer::vsync, gs/gs_renderer.cpp:4189-5055):
 * the display mode from SMODE1/SMODE2, both circuits per PMODE/DISPFB/DISPLAY,
 * merged over BGCOLOR with ALP or circuit-1 alpha, the EXTWRITE write-back into
 * VRAM, and a FastMAD deinterlace of interlaced output.  dst receives
 * result->width x result->height RGBA8; when dst_size is too small nothing
 * runs and PGS_ERROR_CAPACITY is returned with *result filled in.  An unknown
 * video mode returns PGS_OK with a 0 x 0 image. */
#define PGS_VSYNC_FORCE_PROGRESSIVE 1u
#define PGS_VSYNC_HIGH_RESOLUTION 2u
#define PGS_VSYNC_OVERSCAN 4u
#define PGS_VSYNC_CRTC_OFFSETS 8u
#define PGS_VSYNC_ANTI_BLUR 16u
#define PGS_VSYNC_ADAPT_HORIZONTAL 32u
#define PGS_VSYNC_RAW_CIRCUIT 64u
#define PGS_VSYNC_SKIP_DEINTERLACE 128u
/* Largest image pgs_gs_vsync writes (1920 x 1080 doubled by high-resolution
 * read-out). */
#define PGS_VSYNC_MAX_BYTES (3840ull * 2160ull * 4ull)

typedef struct pgs_vsync_info
{
	uint32_t phase; /* field, 0 or 1 */
	uint32_t flags; /* PGS_VSYNC_* */
} pgs_vsync_info;

typedef struct pgs_scanout_result
{
	uint32_t width, height; /* image written to dst */
	uint32_t mode_width, mode_height;
	uint32_t internal_width, internal_height;
	uint32_t interlaced, interlace_phase, double_strike, high_resolution_scanout;
	float sampling_rate_mhz;
	uint32_t padding;
} pgs_scanout_result;

int pgs_gs_vsync(pgs_gs *gs, const pgs_vsync_info *info, void *dst, uint64_t dst_size, pgs_scanout_result *result);
/* GSInterface::vsync_can_skip (gs/gs_interface.cpp:4692-4695): 1 when the
 * read-out is progressive (no field alternation) and no SCANMSK primitive
 * taller than 400 rows was drawn within the last 4 vsyncs, else 0. */
int pgs_gs_vsync_can_skip(const pgs_gs *gs, const pgs_vsync_info *info);
/* GSInterface::map_vram_write + end_vram_write. */
int pgs_gs_write_vram(pgs_gs *gs, uint64_t offset, uint64_t size, const void *src);
/* GSInterface::read_transfer_fifo. */
int pgs_gs_read_transfer_fifo(pgs_gs *gs, void *data, uint32_t num_128b_words);
/* GSInterface::consume_flush_stats. */
int pgs_gs_consume_flush_stats(pgs_gs *gs, pgs_flush_stats *stats);
/* GSInterface::set_super_sampling_rate. */
int pgs_gs_set_super_sampling_rate(pgs_gs *gs, uint32_t super_sampling, uint32_t ordered_grid);
/* The super_sampled_textures argument of set_super_sampling_rate
 * (gs/gs_interface.hpp:258): sprites sampling pages a super-sampled pass wrote
 * read per-sample texture layers.  Ignored at 1x. */
int pgs_gs_set_super_sampled_textures(pgs_gs *gs, int enable);

/* Hacks (gs/gs_interface.hpp:209-237, GSInterface::set_hacks): inaccurate
 * options, all off by default.  disable_mipmaps samples level 0 only;
 * allow_blend_demote sets pgs_render_pass.blend_demote; unsynced_readbacks is
 * accepted and has no effect (FIFO readbacks here always wait for the
 * rendering they read); backbuffer_promotion is not supported and returns
 * PGS_ERROR_UNSUPPORTED. */
typedef struct pgs_hacks
{
	uint32_t disable_mipmaps;
	uint32_t unsynced_readbacks;
	uint32_t backbuffer_promotion;
	uint32_t allow_blend_demote;
} pgs_hacks;
int pgs_gs_set_hacks(pgs_gs *gs, const pgs_hacks *hacks);

/* GSInterface::reset_context_state (gs/gs_interface.cpp:26-39): flushes, then
 * returns the register file, the GIF paths and the vertex queue to their
 * power-on state (PRMODECONT.AC = 1, everything else 0). */
int pgs_gs_reset_context_state(pgs_gs *gs);
/* GSInterface::clobber_register_state (gs/gs_interface.cpp:4266-4274): state
 * derived from registers is rebuilt on the next use, for callers that changed
 * registers behind the interface (pgs_gs_set_register). */
int pgs_gs_clobber_register_state(pgs_gs *gs);
/* get_register_state (gs/gs_interface.hpp:287-288): the register file by A+D
 * address (0x00-0x7f).  pgs_gs_set_register stores a value without the side
 * effects of pgs_gs_write_register (no transfer, kick or flush); follow it with
 * pgs_gs_clobber_register_state. */
int pgs_gs_read_register(const pgs_gs *gs, uint32_t addr, uint64_t *value);
int pgs_gs_set_register(pgs_gs *gs, uint32_t addr, uint64_t value);

/* GIFPath (gs/gs_interface.hpp:63-68, get_gif_path :293-294): the current
 * GIFtag of a path, the register index within a loop and the loops done. */
typedef struct pgs_gif_path
{
	uint64_t tag[2];
	uint32_t reg;
	uint32_t loop;
} pgs_gif_path;
int pgs_gs_get_gif_path(const pgs_gs *gs, uint32_t path, pgs_gif_path *out);
int pgs_gs_set_gif_path(pgs_gs *gs, uint32_t path, const pgs_gif_path *in);

/* SignalInterface (gs/gs_interface.hpp:238-248, set_signal_interface): called
 * for SIGNAL, FINISH and LABEL register writes with the written value; a
 * non-zero return flushes (rendering is submitted, nothing waits).  A NULL
 * interface, or a NULL member, ignores the register. */
typedef int (*pgs_signal_fn)(void *user, uint64_t payload);
typedef struct pgs_signal_interface
{
	pgs_signal_fn on_signal;
	pgs_signal_fn on_finish;
	pgs_signal_fn on_label;
	void *user;
} pgs_signal_interface;
int pgs_gs_set_signal_interface(pgs_gs *gs, const pgs_signal_interface *iface);

/* DebugMode (gs/gs_interface.hpp:137-153, set_debug_mode).  timestamps turns
 * per-stage GPU timing on in a backend that has it (pgs_backend_ops.timestamps);
 * the other members are debugging aids of the Vulkan renderer (render-target
 * feedback, deterministic timeline queries, sampler feedback, per-draw
 * stepping), accepted and without effect here. */
typedef struct pgs_debug_mode
{
	uint32_t feedback_render_target;
	uint32_t timestamps;
	uint32_t deterministic_timeline_query;
	uint32_t disable_sampler_feedback;
	uint32_t draw_mode; /* 0 none, 1 strided, 2 full */
} pgs_debug_mode;
int pgs_gs_set_debug_mode(pgs_gs *gs, const pgs_debug_mode *mode);
/* GSInterface::get_accumulated_timestamps (gs/gs_interface.cpp:4702-4705):
 * seconds of GPU time spent in stage `type` (PGS_TIMESTAMP_*) while timing
 * was on; 0 when the backend does not time stages. */
int pgs_gs_get_accumulated_timestamps(pgs_gs *gs, uint32_t type, double *seconds);

#ifdef __cplusplus
}
#endif

#endif
