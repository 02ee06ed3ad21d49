/*
 * nebc7_gb300 -- BC7 block encoder for NVIDIA GB300 (sm_103a), C ABI.
 *
 * Drop-in for the block compressor of andrewevstyukhin/nebc7: every 128-bit
 * block it writes is bit-identical to the reference CPU encoder's for the
 * same input, mask, starting blocks, preset and flags.
 *
 * Two layers:
 *
 *  1. The reference's own interfaces, as plain C:
 *       nebc7_GetBc7Core      fills an IBc7Core vtable
 *                             (reference src/Bc7Core.h:316-322, src/Bc7Core.cpp:1998);
 *       nebc7_ProcessTexture  whole-texture job entry
 *                             (reference src/Worker.h:6, src/Worker.cpp:249).
 *     The reference passes its error accumulators by C++ reference; here they
 *     are pointers (the same machine-level ABI).  The reference fixes
 *     kDenoise / kDenoiseStep at compile time (src/Bc7Mode.h:10-13); here
 *     nebc7_set_preset selects them at run time.
 *
 *  2. Direct entries on device or host buffers (nebc7_encode_*,
 *     nebc7_decode_*), with explicit settings and CUDA streams.
 *
 * All functions return 0 on success or one of the NEBC7_E* codes.  The
 * IBc7Core kernels have no error channel (the reference's are noexcept);
 * they leave their outputs untouched on failure and record the code for
 * nebc7_last_error().
 */
#ifndef NEBC7_GB300_H
#define NEBC7_GB300_H

#include <stdbool.h>
#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

enum
{
	NEBC7_OK = 0,
	NEBC7_EINVAL = 1,        /* bad argument (sizes, alignment, preset) */
	NEBC7_ECUDA = 2,         /* a CUDA call failed */
	NEBC7_ENOMEM = 3,        /* device memory could not be allocated */
	NEBC7_EUNSUPPORTED = 4,  /* requested pass not compiled into the library */
	NEBC7_ELIMIT = 5,        /* a device-side iteration limit was reached */
	NEBC7_ETOOBIG = 6        /* request exceeds a fixed capacity */
};

/* ---- reference block API (src/Bc7Core.h:294-322) ---------------------- */

typedef struct WorkerItem
{
	uint8_t* _Output;   /* 16 bytes: starting block in, encoded block out */
	uint8_t* _Cell;     /* 4 rows of 4 BGRA pixels, `stride` bytes apart */
	uint8_t* _Mask;     /* 4 rows of 4 masks (bytes A,G,R,B), same stride */
} WorkerItem;

typedef struct BlockSSIM
{
	double Alpha, Color;
} BlockSSIM;

typedef void (*PInitTables)(bool doDraft, bool doNormal, bool doSlow, bool linearData);
typedef void (*PBlockKernel)(const WorkerItem* begin, const WorkerItem* end, int stride,
	int64_t* pErrorAlpha, int64_t* pErrorColor, BlockSSIM* pssim);
typedef int (*PGetWeight)(void);

typedef struct IBc7Core
{
	PInitTables pInitTables;
	PBlockKernel pDecompress, pCompress;
	PGetWeight pGetWeightAlpha, pGetWeightColor;
} IBc7Core;

/* Replaces GetBc7Core (src/Bc7Core.cpp:1998): fills the vtable; false if no
   usable CUDA device is present.  pInitTables (src/Bc7Core.cpp:1877) stores
   the flags and weights and builds the level tables of the current preset
   on the current device.  pCompress (src/Bc7Core.cpp:1936) encodes the items
   on the GPU and *adds* Error.Alpha << 2kD, (Error.Total - Error.Alpha) <<
   2kD and the SSIM values to the accumulators, as the reference does.
   pDecompress (src/Bc7Core.cpp:1904) writes the decoded BGRA rows to _Cell. */
bool nebc7_GetBc7Core(void* bc7Core);

/* Replaces ProcessTexture (src/Worker.h:6): splits the padded texture
   (src_w, src_h multiples of 4) into 4x4 blocks and runs `blockKernel`
   (pCompress or pDecompress of this library) on all of them in one launch.
   Host buffers; block_size must be 16.  Accumulators are assigned, like the
   reference's Worker::Run. */
void nebc7_ProcessTexture(uint8_t* dst, uint8_t* src_bgra, uint8_t* mask_agrb, int stride, int src_w, int src_h,
	PBlockKernel blockKernel, size_t block_size, int64_t* pErrorAlpha, int64_t* pErrorColor, BlockSSIM* pssim);

/* The compile-time preset of the reference (src/Bc7Mode.h:10-13) chosen at
   run time: denoise (kDenoise) 0 or 1, denoiseStep (kDenoiseStep) >= 0.
   Default 1, 9.  Takes effect for later calls. */
int nebc7_set_preset(int denoise, int denoiseStep);

/* Last error recorded by a call without an error channel. */
int nebc7_last_error(void);

/* ---- direct entries ----------------------------------------------------- */

typedef struct nebc7_settings
{
	int denoise;        /* kDenoise: 0 or 1 */
	int denoiseStep;    /* kDenoiseStep */
	int doDraft;        /* bounding-box passes (the CLI always sets this); 2: only the
	                       Mode6Index2 pass (the "Mode6Index2 fast" run, no refinement;
	                       no counterpart in the reference) */
	int doNormal;       /* refinement + full searches of modes 2, 0 / 5, 4, 7 */
	int doSlow;         /* full searches of every mode */
	int linearData;     /* /data: equal channel weights */
} nebc7_settings;

/* Encodes a padded texture (w, h multiples of 4) on the GPU.  Device
   pointers: d_dst holds w*h/16 blocks (16-byte aligned), read as the starting
   blocks (all-zero bytes = start from scratch) and overwritten; d_bgra / d_mask
   hold rows of w pixels `stride` bytes apart (4-byte aligned); d_mask may be
   null for a full mask.  `stream` is a cudaStream_t (null = default).
   If errs / ssim are non-null the call waits for the stream and stores the
   error sums (alpha, color) and SSIM sums there; otherwise it only enqueues. */
int nebc7_encode_device(uint8_t* d_dst, const uint8_t* d_bgra, const uint8_t* d_mask, long long stride, int w, int h,
	const nebc7_settings* settings, int64_t* errs, double* ssim, void* stream);

/* Same with host buffers: copies in, encodes, copies the blocks back, and
   waits.  Device staging buffers are cached per device and per concurrent
   caller for the life of the process (they only grow), so repeated calls do
   not allocate; pinned host buffers give the fastest copies.  Safe to call
   from several threads at once. */
int nebc7_encode_host(uint8_t* dst, const uint8_t* bgra, const uint8_t* mask, long long stride, int w, int h,
	const nebc7_settings* settings, int64_t* errs, double* ssim);

/* Independent blocks: cells / masks hold 64 bytes per block (4 rows of 4
   pixels), io 16 bytes per block (starting block in, result out).  Host
   buffers. */
int nebc7_encode_blocks_host(const uint8_t* cells, const uint8_t* masks, uint8_t* io, int n,
	const nebc7_settings* settings, int64_t* errs, double* ssim);

/* Decodes blocks to BGRA (device pointers; rows of w pixels, `stride`
   bytes apart). */
int nebc7_decode_device(const uint8_t* d_blocks, uint8_t* d_bgra, long long stride, int w, int h, void* stream);

/* Decodes n blocks to 64 bytes of BGRA each (host buffers). */
int nebc7_decode_blocks_host(const uint8_t* blocks, uint8_t* bgra, int n);

/* OPTION_PCA (src/Bc7Mode.h:5, off in the reference's build and here by
   default): the full searches of modes 1, 3, 6 and 7 order and bound their
   partitions by the principal-axis residual of each area
   (PrincipalComponentAnalysis, src/Bc7PcaEigen.cpp:26-146; consumers
   src/Bc7Core.cpp:494, src/Bc7CoreMode1.cpp:490-496, Mode3.cpp:488-494,
   Mode6.cpp:1383-1396, Mode7.cpp:559-572).  Applies to encodes, batches and
   servers created after the call.  The reference takes the axis from the
   third-party Eigen 3.3.7, absent from its tree; the SVD here restates
   Eigen's published JacobiSVD, so PCA-on outputs are not pinned to a PCA
   build of the reference (they are tested against the CPU restatement). */
int nebc7_set_pca(int on);

/* How many kernels one nebc7_encode_device call with these settings
   launches (the block order, then the encode: one persistent kernel, or
   for the presets whose time goes to the full searches the staged form of
   a kernel per pass and a list kernel before each, the split passes with a
   task and a commit kernel per round), not counting the sums' reduction;
   a negative error code for invalid settings. */
int nebc7_encode_launches(const nebc7_settings* settings);

/* Builds the level tables of `denoise` on the current device ahead of use. */
int nebc7_init_device(int denoise);

/* Copies level table `which` (0..14, in the order d2v8, d2v7, d2v6, d2v5,
   c2v8, c2v6, c2v5, d3v7s, d3v6, d3v5, c3v7s, c3v5, d4h, d2h, d3v8) of `denoise`
   from the current device to `host`, building the tables first if needed.
   *bytes receives the table's size; NEBC7_ETOOBIG when `capacity` is
   smaller.  The reference's tables are process globals filled by
   InitLevels (src/Bc7Tables.cpp:583-777); this read-back lets a caller
   compare the device-built copies with them entry by entry.  d2v8, d4h and
   d2h are stored by endpoint differences here: [cH - x + 255][cL - x + 255],
   511 rows of 512 bytes or of 256 bytes of packed nibbles.  d3v8 has no
   reference counterpart: the byte table of 3-bit indices with 8-bit
   endpoints, by differences, which the encoder reads in place of the
   reference's reduced tables of 3-bit indices (their entries at the
   bit-replicated endpoints). */
int nebc7_table_read(int denoise, int which, void* host, long long capacity, long long* bytes);

/* Allocation-free variant of nebc7_encode_device (no counterpart in the
   reference, whose CPU encoder needs no device memory).  For callers that
   cannot let the library allocate device memory while they run: a serving
   loop that admits jobs against a fixed HBM budget, or a loop that must not
   meet the device-wide synchronisation cudaMalloc / cudaFree can cause.
   The call itself makes no allocation of any kind.  Its scratch is one
   fixed device array inside the library, sized for at most 65536 blocks
   (a 1024x1024 texture); larger textures are rejected with NEBC7_ETOOBIG.
   Setup: call nebc7_init_device(settings->denoise) on the device first (it
   allocates the level tables; without it this call returns NEBC7_EINVAL).
   The first call on each device does one-time setup with that device
   current (it looks up the scratch array's address and sizes the kernel's
   launch); make that first call before any stream capture.
   Each call zeroes the scratch's work-queue head and status word on
   `stream` before its kernel; nothing else needs to start at zero.
   d_sums, if non-null (8-byte aligned device memory), receives
   { int64 errAlpha, int64 errColor, double ssimAlpha, double ssimColor }
   as nebc7_encode_device reports them.  The call only enqueues work and
   never waits.  All calls on a device share the one scratch array, so calls
   whose work overlaps on the device (different streams, or threads without
   ordering) race and corrupt each other's results: issue them in one stream
   or order them. */
int nebc7_encode_device_noalloc(uint8_t* d_dst, const uint8_t* d_bgra, const uint8_t* d_mask, long long stride, int w,
	int h, const nebc7_settings* settings, void* d_sums, void* stream);

/* ---- batches (no counterpart in the reference) ------------------------- */

/* One texture of a batch: device buffers as for nebc7_encode_device. */
typedef struct nebc7_texture
{
	uint8_t* d_dst;            /* w*h/16 blocks, 16-byte aligned: starting blocks in, result out */
	const uint8_t* d_bgra;     /* padded BGRA rows, `stride` bytes apart */
	const uint8_t* d_mask;     /* mask rows (A,G,R,B bytes) or null */
	long long stride;
	int w, h;                  /* multiples of 4 */
	nebc7_settings settings;   /* the texture's own preset and flags */
} nebc7_texture;

typedef struct nebc7_batch nebc7_batch;

#define NEBC7_BATCH_FROM_SCRATCH 1   /* every launch clears the outputs first */

/* Plans a batch of textures of any sizes and presets: one persistent
   kernel launch over a global block queue (textures of the longest
   expected work first), or one such launch per preset group on concurrent
   streams.  Allocates the plan's device tables and scratch (per-block
   results, per-texture sums) on the current device; the textures' buffers
   stay the caller's and must outlive the plan. */
int nebc7_batch_create(const nebc7_texture* textures, int n, int flags, nebc7_batch** out);

/* Tunes the plan (nebc7_batch_trials lists the search): each candidate is
   replayed `trials` times as a CUDA graph and the fastest is kept for
   nebc7_batch_launch; restores the starting blocks afterwards unless the
   plan clears them itself.  ms_out[2], if non-null, receives the best times
   of the mixed and the grouped schedule (3.4e38 if not tried). */
int nebc7_batch_tune(nebc7_batch* b, int trials, float* ms_out);

/* Enqueues the batch on `stream` by replaying its CUDA graph (captured on
   the first call for the chosen schedule).  Outputs and sums are ready
   when the stream reaches this point. */
int nebc7_batch_launch(nebc7_batch* b, void* stream);

/* Copies the per-texture sums of the last launch (errs[2 i] = Error.Alpha
   << 2kD, errs[2 i + 1] = color part, ssim[2 i], ssim[2 i + 1]; either may
   be null) after waiting for `stream`. */
int nebc7_batch_sums(nebc7_batch* b, void* stream, int64_t* errs, double* ssim);

/* Overrides the schedule: 0 one mixed launch, 1 one launch per preset group. */
int nebc7_batch_set_schedule(nebc7_batch* b, int schedule);

/* The plan's knobs: the schedule (0 mixed, 1 grouped), whether the groups
   whose presets run the full searches use the staged form (one kernel per
   pass; 1) or one kernel (0), and the resident CTAs per SM of the
   persistent launches (0: as many as fit).  nebc7_batch_set_plan drops the
   captured graphs when the staged form or the CTAs change. */
int nebc7_batch_plan(const nebc7_batch* b, int* schedule, int* staged, int* ctas_per_sm);
int nebc7_batch_set_plan(nebc7_batch* b, int schedule, int staged, int ctas_per_sm);

/* The plans the last nebc7_batch_tune timed, in order, with their best ms
   (arrays of cap entries, any may be null); returns how many there were.
   The tuner starts from one mixed launch, staged, at full occupancy, and
   keeps each change that is faster: the grouped schedule, then one kernel
   per group, then 2 CTAs per SM. */
int nebc7_batch_trials(const nebc7_batch* b, int* schedule, int* staged, int* ctas_per_sm, float* ms, int cap);

/* Chosen schedule (0 mixed, 1 grouped), kernel launches per run, blocks. */
int nebc7_batch_info(const nebc7_batch* b, int* schedule, int* launches, int* blocks);

void nebc7_batch_destroy(nebc7_batch* b);

/* ---- serving (no counterpart in the reference) ------------------------- */

typedef struct nebc7_server nebc7_server;

typedef struct nebc7_server_config
{
	size_t hbm_budget;   /* device bytes for requests in flight (sources, masks, outputs, per-block results) */
	int max_batch;       /* requests per launch */
	int streams;         /* launches in flight at once */
} nebc7_server_config;

typedef struct nebc7_request_info
{
	int status;          /* NEBC7_OK or the error of the request */
	double queue_ms;     /* submit -> its launch was enqueued */
	double latency_ms;   /* submit -> its blocks were back in host memory */
	int64_t errs[2];     /* as nebc7_encode_host reports them */
	double ssim[2];
	/* when it was submitted, launched and back in host memory (ms since the
	   server's creation), the launch slot and the launch's sequence number:
	   requests of different launches whose [launch_at, done_at] spans
	   overlap ran on the device at the same time */
	double submit_at_ms, launch_at_ms, done_at_ms;
	int slot;
	long long launch;
} nebc7_request_info;

typedef struct nebc7_server_counters
{
	long long completed, failed, launches, queued, bytes_in_use, peak_bytes;
} nebc7_server_counters;

/* Starts a request loop on the current device: one device arena of
   hbm_budget bytes holds the sources, masks, outputs and per-block results
   of the requests in flight.  A scheduler thread admits requests in
   arrival order while the arena has room, and starts a batch of admitted
   requests on every free stream, so requests that arrive while others run
   join the device as soon as a stream and memory free up.  A batch is the
   oldest admitted request and later ones of its kind: heavy presets (the
   precise preset, /slow, /data) run as one staged launch (a kernel per
   pass), light ones as one persistent launch with presets mixed, the
   cheapest requests dealt first; each request of a light batch returns
   (its blocks copied back) as soon as its own blocks are done, while the
   rest of the launch still runs.  Besides the arena, every stream holds the
   staged form's per-block state (its record, pass lists, split-pass rounds
   and kept results): 156 bytes per block for up to min(4194304,
   hbm_budget / 104) blocks. */
int nebc7_server_create(const nebc7_server_config* cfg, nebc7_server** out);

/* Queues one texture (host buffers; pinned memory lets the copies run
   asynchronously) to be encoded from scratch into host `dst` (w*h/16
   blocks).  The buffers must stay valid until nebc7_server_wait returns.
   NEBC7_ETOOBIG if the request alone exceeds the budget. */
int nebc7_server_submit(nebc7_server* s, const uint8_t* bgra, const uint8_t* mask, long long stride, int w, int h,
	const nebc7_settings* settings, uint8_t* dst, int64_t* ticket);

/* Waits for a request (timeout_s < 0: without limit; NEBC7_ELIMIT on
   timeout, the ticket stays valid), fills `info` and releases the ticket. */
int nebc7_server_wait(nebc7_server* s, int64_t ticket, double timeout_s, nebc7_request_info* info);

int nebc7_server_stats(nebc7_server* s, nebc7_server_counters* out);

/* Finishes the queued and running requests, then frees the server. */
void nebc7_server_destroy(nebc7_server* s);

/* ---- the driver's steps around the encode, on the device ---------------- */

/* Pads a w x h BGRA image (rows src_stride bytes apart) to the texture size
   the reference encodes (each side max(4, n) rounded up to 4) by repeating
   the last column and row (src/Bc7Compress.cpp:397-426), into d_padded
   (rows 4 * padded width bytes apart).  If d_mask is non-null it receives
   the mask of the padded texture (same layout, bytes A, G, R, B): the alpha
   outline of the given radius (src/Bc7Compress.cpp:33-105), or all 0xFF for
   radius < 0 (/nomask). */
int nebc7_prepare_device(const uint8_t* d_src, long long src_stride, int w, int h, uint8_t* d_padded, uint8_t* d_mask,
	int radius, void* stream);

/* The /bad glitch map (src/Worker.cpp:309-451): for each block whose decoded
   pixels differ from the source by at least 16 / 12 / 16 / 20 (A, G, R, B;
   16 each with linear weights) in a masked channel, d_out gets the source
   pixels; other blocks are cleared.  Padded textures, one stride. */
int nebc7_bad_blocks_device(const uint8_t* d_src, const uint8_t* d_decoded, const uint8_t* d_mask, long long stride, int w, int h,
	int linear, uint8_t* d_out, void* stream);

/* The /map partition visualisation (src/Bc7Compress.cpp:131-265): rewrites
   blocks so that decoding them (nebc7_decode_device) shows each block's
   mode and partition as flat colours. */
int nebc7_partition_map_device(const uint8_t* d_blocks, uint8_t* d_out, int nblocks, void* stream);

/* The 96-byte KTX 1.1 header the reference writes before the blocks of a
   w x h image (src/Bc7Compress.cpp:439-463); flip selects the orientation
   key "T=u" (bottom-up rows) instead of "T=d". */
int nebc7_ktx_header(int w, int h, int flip, uint8_t* out);

/* Persistent-grid sizing of the encode kernel of the default preset
   (kDenoise 1 with the refinement passes): CTAs per SM and warps per CTA. */
int nebc7_launch_shape(int* ctas_per_sm, int* warps_per_cta, int* sm_count);

#ifdef __cplusplus
}
#endif

#endif /* NEBC7_GB300_H */
