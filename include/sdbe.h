/*
 * sdbe.h -- C ABI of the GB300 SWARM->R2DBE resampling stage.
 *
 * Drop-in for the GPU stage of APHIDS in Smithsonian/sdbe:
 *   software/aphids/vdif_inout_gpu_thread.cu (hashpipe thread "VDIFIO",
 *   .cu:1047-1059) with its buffer layouts from vdif_in_databuf.h and
 *   vdif_out_databuf.h.  Every entry point is plain C: pointers, sizes and
 *   int status codes; nothing aborts.  Device pointers live on the device the
 *   handle was created for.  "stream" arguments are cudaStream_t values passed
 *   as void* (NULL = the handle's own stream, or the legacy default stream for
 *   handle-less calls).
 *
 * Layouts (byte-compatible with the reference):
 *   input packet  : 1056 B = 32 B VDIF header + 1024 B payload
 *                   (vdif_in_packet_t, vdif_in_databuf.h:29-67); B-engine
 *                   counter b = (w4 << 8) | (w5 >> 24), c = w5 & 0xFF,
 *                   f = (w5 >> 16) & 0xFF.
 *   output payload: [2 pols][n_batches*128 packets][8192 B], 16 two-bit
 *                   samples per little-endian u32, sample i at bits 2i..2i+1
 *                   (vdif_out_data_group_t, vdif_out_databuf.h:110-116).
 *   output frame  : 8224 B = 32 B header + 8192 B payload (vdif_out_packet_t).
 */
#ifndef SDBE_H
#define SDBE_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes (reference: STATE_PROC=1 / STATE_ERROR=-1, .cu:37-39) -- */
#define SDBE_OK 0
#define SDBE_ERR_ARG -1        /* bad argument or size                      */
#define SDBE_ERR_CUDA -2       /* a CUDA runtime call failed                */
#define SDBE_ERR_STATE -3      /* call not valid in the handle's state      */
#define SDBE_ERR_CAPACITY -4   /* input or output larger than configured    */
#define SDBE_ERR_NOMEM -5      /* device or host allocation failed          */

/* ---- constants of the SWARM 11/11 build (sample_rates.h, .h:10-53) ------- */
#define SDBE_IN_PKT_BYTES 1056
#define SDBE_OUT_PKT_DATA_BYTES 8192
#define SDBE_OUT_PKT_BYTES 8224
#define SDBE_PKTS_PER_FRAME 2048
#define SDBE_SNAPSHOTS_PER_FRAME 128
#define SDBE_CHANNELS 16384
#define SDBE_BATCH_SNAPSHOTS 143      /* DECIMATION_FACTOR                    */
#define SDBE_PKTS_PER_BATCH 128       /* EXPANSION_FACTOR: out packets/batch  */
#define SDBE_FRAMES_PER_GROUP 143     /* BENG_FRAMES_PER_GROUP                */
#define SDBE_SAMPLES_PER_OUT_PKT 32768
#define SDBE_MAX_SKIP_CHAN 1920       /* 18304 - 16384 bins                    */

/* threshold modes */
#define SDBE_THRESH_FIRST_BATCH 0  /* reference: mean/std of the first batch, set once (.cu:953-986) */
#define SDBE_THRESH_FIXED 1        /* thresholds supplied by sdbe_set_state                          */
/* Windowed thresholds (no counterpart in the reference, which sets them
 * once): batch 0 of the stream sets them as SDBE_THRESH_FIRST_BATCH does;
 * from then on, at every SDBE_THRESH_BLOCK-batch boundary T of the stream,
 * the mean and standard deviation of the FP64 statistics of batches
 * [max(0, T - threshold_window), T) set the thresholds of the next block.
 * The statistics are gathered in the same pass that quantizes (no extra
 * read of the floats); waves are cut at block boundaries, so results do not
 * depend on wave_batches. */
#define SDBE_THRESH_WINDOW 2
#define SDBE_THRESH_BLOCK 16

/* channel maps */
#define SDBE_MAP_APHIDS 0          /* ((c>>1)*16 + (c&1) + 2f)*8, .cu:442                */
#define SDBE_MAP_MAR2015 1         /* 8*(8c + f), prototyping/read_sdbe_vdif.py:193      */

/* arithmetic of the three FFT stages (A: C2R 32768, B: R2C 36608, C: C2R 32768) */
#define SDBE_PRECISION_FP32 0      /* FP32 radix kernels on the CUDA cores (default)     */
/* FP16 tensor cores: each transform a four-step GEMM (tcgen05.mma, FP32
 * accumulation in tensor memory).  TC16 splits the DFT matrix and the data
 * into hi + lo FP16 halves (three products per real product: FP32-like
 * error); TC16_FAST splits only the DFT matrix and rounds the data to FP16
 * (two products).  All entry points and threshold modes. */
#define SDBE_PRECISION_TC16 1
#define SDBE_PRECISION_TC16_FAST 2
#define SDBE_STAGES_FUSED 1
#define SDBE_STAGES_SPLIT 3

/* sdbe_process flags */
#define SDBE_IN_HOST 1u            /* packets are in host memory (copied in)             */
#define SDBE_OUT_HOST 2u           /* output goes to host memory (copied out)            */
#define SDBE_OUT_FRAMED 4u         /* write 8224-B VDIF frames with headers              */
#define SDBE_SYNC 8u               /* synchronize the stream before returning            */
#define SDBE_ASYNC 16u             /* with host buffers: return without waiting; the
                                      buffers must stay valid until sdbe_sync          */
#define SDBE_OUT_ALIGNED 32u       /* time-aligned 8224-B VDIF frames (implies FRAMED):
                                      the output thread's skip + leftover carry         */
#define SDBE_IN_8PAC 64u           /* sdbe_ingest: input is 8pac units with new-format
                                      B-engine headers (unpack + reform first)          */
#define SDBE_PAC8_BYTES 8504       /* sizeof(vdif_8pac_packet_t), vdif_8pac.h:8-16     */

typedef struct sdbe_config {
    int32_t device;            /* CUDA device ordinal (resampler->deviceId, .cu:147)        */
    int32_t trim_mhz;          /* MHz trimmed from DC, Redis key trim_from_dc (.cu:770,269) */
    int32_t max_frames;        /* most B-frames per sdbe_process call (143 = one group)     */
    int32_t threshold_mode;    /* SDBE_THRESH_*                                             */
    int32_t pol1_uses_pol0_threshold; /* 1 reproduces .cu:1004-1005 (pol 1 quantized with
                                         pol 0's threshold/offset); 0 = each pol its own    */
    int32_t channel_map;       /* SDBE_MAP_*                                                */
    int32_t wave_batches;      /* batches per FFT wave, 1..64; 0 = 64, or fewer when       */
                               /* max_frames cannot fill 64; scratch 37.5 MB per batch     */
    int32_t threshold_window;  /* SDBE_THRESH_WINDOW: batches in the window (0 = 64)        */
    int32_t precision;         /* SDBE_PRECISION_*                                          */
    int32_t stage_launches;    /* SDBE_PRECISION_TC16_FAST waves: SDBE_STAGES_FUSED (one
                                  persistent launch runs stages A, B and C on a device work
                                  queue) or SDBE_STAGES_SPLIT (a launch per stage); 0 =
                                  SDBE_STAGES_FUSED.  Other precisions ignore it.          */
    int32_t reserved[6];
} sdbe_config;

typedef struct sdbe_state {
    float threshold[2];        /* quantizeThreshold_0/1 (.cu:151), own value per pol       */
    float offset[2];           /* quantizeOffset_0/1 (.cu:152)                             */
    int32_t thresholds_set;    /* 0 until computed or supplied                             */
    int32_t carry_snapshots;   /* snapshots held for the next call (< 143)                 */
    /* output VDIF header counters (vdif_out_net_thread.c:199-317) */
    uint32_t secs_inre;
    uint32_t df_num_insec;
    uint64_t edh_psn;
    uint32_t ref_epoch;
    uint32_t station_id;
    uint32_t bdc_sideband;
    uint32_t rx_sideband;
    int32_t reserved[6];
} sdbe_state;

typedef struct sdbe_result {
    int64_t n_batches;         /* 143-snapshot batches processed                            */
    int64_t n_out_packets;     /* output packets per pol (= 128 * n_batches)                */
    int64_t packets_accepted;  /* scattered into the group                                  */
    int64_t packets_rejected;  /* invalid flag, f >= 8 or b outside the window              */
    int64_t frames_incomplete; /* frames with fewer than 2048 distinct (c,f) packets        */
    int64_t carry_snapshots;
} sdbe_result;

typedef struct sdbe_resampler sdbe_resampler;

/* Create: device buffers, twiddle tables, stream.
 * Replaces aphids_resampler_init (vdif_inout_gpu_thread.cu:184-347). */
int sdbe_create(const sdbe_config *cfg, sdbe_resampler **out);

/* Destroy: frees everything the handle owns.
 * Replaces aphids_resampler_destroy (.cu:712-743); does not reset the device. */
int sdbe_destroy(sdbe_resampler *h);

/* Output payload bytes one sdbe_process call on n_frames B-frames writes
 * (both pols), given the current carry; frames with flag SDBE_OUT_FRAMED use
 * 8224-B slots.  Lets the caller size its buffer. */
int64_t sdbe_output_bytes(const sdbe_resampler *h, int32_t n_frames, uint32_t flags);

/* Process n_frames consecutive B-frames of packets starting at counter b_zero
 * (packet order arbitrary, missing packets read as zero).
 * Replaces one pass of run_method's STATE_PROC body (.cu:874-1017): the
 * vdif_to_beng unpack (K1, .cu:894-906), then per 143-snapshot batch
 * beng_int8_to_cufftComplex, SwarmC2R, SwarmR2C, R2dbeC2R, the one-off
 * threshold and quantize2bit (.cu:923-1008).  With n_frames = 143 and no
 * carry the output is exactly vdif_out_data_group_t.
 *   packets   : n_packets*1056 B, host (SDBE_IN_HOST) or device memory
 *   out       : host (SDBE_OUT_HOST) or device; out_bytes = its capacity
 *   result    : optional; filling it synchronizes the stream
 * With SDBE_OUT_FRAMED the headers come from the handle's header counters,
 * which advance by the packets written.
 * Host buffers go through two device staging slots on separate copy streams:
 * the payloads of each FFT wave leave for the host while the next wave
 * computes, and with SDBE_ASYNC the next call's packet upload overlaps this
 * call's compute (the overlap the reference gets from its separate ingest,
 * GPU and output threads).  Host buffers should be pinned (sdbe_host_alloc). */
int sdbe_process(sdbe_resampler *h, const void *packets, int64_t n_packets, int32_t n_frames,
                 uint64_t b_zero, void *out, int64_t out_bytes, uint32_t flags, void *stream,
                 sdbe_result *result);

/* State of the stream.  get/set synchronize the device first (work may be in
 * flight on any stream).  set: thresholds/offsets (marked set if any
 * threshold != 0), header counters; clears the carry when carry_snapshots == 0. */
/* Output time alignment (vdif_out_net_thread.c:199-317, template from
 * fill_vdif_header_template, vdif_in_databuf.c:193-220).  A template holds
 * the first output second, data frame and the picoseconds the stream starts
 * early.  sdbe_align_start arms it for the next SDBE_OUT_ALIGNED call, which
 * starts on the next second boundary if its block would cross one, skips
 * floor(floor((ps + 3715791) * 4096e6 / 1e12) / 16) payload words and sets psn
 * to 1.  Every aligned call frames whole 8192-B packets of the word stream
 * (previous call's leftover words, then this call's) and carries the rest, so
 * its packet count is floor((leftover + words) / 2048) per pol
 * (sdbe_result.n_out_packets). */
typedef struct sdbe_time_template {
    uint32_t secs_inre;
    uint32_t df_num_insec;
    uint64_t ps_early;         /* edh_psn field of the reference template */
    uint32_t ref_epoch;
    uint32_t reserved;
} sdbe_time_template;
/* Template from the first B-engine timestamp (t0_sec, t0_clk at 286 MHz). */
int sdbe_header_template(int32_t t0_sec, int32_t t0_clk, uint32_t ref_epoch, sdbe_time_template *out);
int sdbe_align_start(sdbe_resampler *h, const sdbe_time_template *t);

/* Group assembly: packets as received from the network, restating the
 * ingest thread (vdif_in_net_thread.c:255-500, vdif_in_databuf.c:96-167).
 * Each batch is sorted invalid-first then by B-counter; the first valid b of
 * the stream fixes groups of 143 B-frames starting at b_first + 1; a ring of
 * 4 open groups takes packets (at most 2048 per frame, 292864 per group); a
 * packet more than 2 groups ahead of the oldest open group ships that group
 * incomplete (missing packets read as zero); a complete group ships at once;
 * packets before the oldest group, more than 4*143 frames beyond the ring,
 * or flagged invalid are counted and dropped.  Every shipped group runs the
 * stage and writes one vdif_out_data_group_t ([2][16384][8192]) to out, in
 * ship order, or with SDBE_OUT_FRAMED [2][16384] 8224-B VDIF frames whose
 * headers continue the handle's counters; *n_groups returns how many.
 * packets are host (SDBE_IN_HOST) or device memory (16-byte aligned, 8-byte
 * for SDBE_IN_8PAC; the policy reads headers produced on the device); out is
 * host (SDBE_OUT_HOST) or 16-byte aligned device memory with room for
 * out_groups groups (otherwise SDBE_ERR_CAPACITY before any change of state,
 * with *n_groups set to the number the batch ships).  Not available with the
 * Mar-2015 channel map. */
typedef struct sdbe_ingest_stats {
    int64_t packets;           /* received                                      */
    int64_t invalid;           /* invalid flag                                  */
    int64_t before_start;      /* b before the oldest open group (skipped)      */
    int64_t too_far_ahead;     /* b more than 4*143 frames beyond the ring      */
    int64_t used;              /* offered to a group                            */
    int64_t overflow;          /* offered but over the frame/group limits       */
    int64_t groups_shipped;
    int64_t groups_incomplete; /* shipped with fewer than 292864 packets        */
    int64_t b_first;           /* -1 until the first valid packet               */
    int64_t reserved[3];
} sdbe_ingest_stats;
int sdbe_ingest(sdbe_resampler *h, const void *packets, int64_t n_packets, void *out, int64_t out_groups,
                uint32_t flags, int32_t *n_groups);
/* Ship every open group that holds packets (end of stream; the reference
 * drops them instead). */
int sdbe_ingest_flush(sdbe_resampler *h, void *out, int64_t out_groups, uint32_t flags, int32_t *n_groups);
int sdbe_ingest_get_stats(const sdbe_resampler *h, sdbe_ingest_stats *st);

/* Ingest transforms (vdif_in_net_thread.c:291-298), the receive-side
 * pre-pass for SWARM's 8pac output.
 *
 * sdbe_unpack_8pac: n_units 8504-B units -> 8*n_units 1056-B packets, device
 * memory, 8-byte aligned (unpack_8pac, vdif_8pac.c:47-56): df_len of all 8 set
 * to ((df_len_1 - 7)/8) & 0xFFFFFF, df_num_insec 8*df_1 + k, psn 8*psn_1 + k,
 * packet 1's invalid flag copied to the other 7, VTP prefixes dropped.  Unlike
 * the reference, the input units are left unmodified.
 *
 * sdbe_beng_reform: rewrite new-format B-engine headers (a 53-bit SWARM
 * timestamp, c, 3-bit f) to the old format in place on the device, with the
 * B-count = frames since the first valid packet (beng_reform_headers,
 * beng_reform.c:137-186).  The reference keeps T0/TPREV/BPREV in file-scope
 * statics; here they are the caller's sdbe_reform_state (start from
 * sdbe_reform_init), read and written by each call, which synchronizes the
 * stream.  sdbe_header_template(t0_sec, t0_clk, ...) takes T0 from it
 * (get_beng_t0, beng_reform.c:113-126, applies the one-frame correction). */
typedef struct sdbe_reform_state {
    int32_t t0_sec, t0_clk;       /* first valid packet's timestamp; -1, -1 until then      */
    int32_t tprev_sec, tprev_clk; /* last counted packet's timestamp (TPREV)                */
    int64_t bprev;                /* its B-count (BPREV; a 32-bit int in the reference)     */
    int64_t marked_invalid;       /* packets invalidated for a jump beyond 1000 frames      */
    int64_t slow_tiles;           /* 1024-packet tiles counted one packet at a time         */
    int64_t reserved;
} sdbe_reform_state;
int sdbe_reform_init(sdbe_reform_state *st);
int sdbe_unpack_8pac(const void *src, int64_t n_units, void *dst, void *stream);
int sdbe_beng_reform(sdbe_reform_state *st, void *pkts, int64_t n_pkts, void *stream);
/* The reform state of a handle's sdbe_ingest stream (SDBE_IN_8PAC batches). */
int sdbe_ingest_reform_state(const sdbe_resampler *h, sdbe_reform_state *st);

/* Several packet streams in one pass: each handle keeps its own state
 * (thresholds, carry, header counters, alignment) and its own descriptor, as
 * if sdbe_process were called on each in turn, but the FFT work of all of
 * them runs in shared launches: the first-batch threshold path of every
 * handle that needs it in one pair of launches, then waves in which one
 * stage-A and one stage-BC launch cover every handle's next batches (wave =
 * the smallest wave_batches of the handles).  Outputs equal the per-handle
 * calls bit for bit.  1 <= n <= 32 distinct handles on one device; flags and
 * stream apply to all (NULL: the first handle's stream); results (optional)
 * has n entries.  Every descriptor is checked before any work is queued.
 * With device buffers, no SDBE_SYNC/ASYNC and results NULL, the call issues
 * only stream-ordered work on `stream` and can be captured into a CUDA graph
 * (the handles' host-side state advances once, at capture). */
typedef struct sdbe_stream_desc {
    const void *packets;
    int64_t n_packets;
    int32_t n_frames;
    int32_t reserved;
    uint64_t b_zero;
    void *out;
    int64_t out_bytes;
} sdbe_stream_desc;
int sdbe_process_multi(sdbe_resampler *const *handles, const sdbe_stream_desc *descs, int32_t n, uint32_t flags,
                       void *stream, sdbe_result *results);

/* Wait for all work the handle issued (its streams and the last stream passed
 * to sdbe_process). */
int sdbe_sync(sdbe_resampler *h);
int sdbe_get_state(sdbe_resampler *h, sdbe_state *st);
int sdbe_set_state(sdbe_resampler *h, const sdbe_state *st);
/* Forget thresholds and carry (a new stream).  Host-side only: the next
 * sdbe_process recomputes the thresholds on its stream, so this is safe while
 * earlier calls are still running. */
int sdbe_reset(sdbe_resampler *h);

/* Per-stage GPU timing, the counterpart of the reference's GPU_DEBUG event
 * timing (vdif_inout_gpu_thread.cu:594-621).  While enabled, sdbe_process
 * records CUDA events around every stage-A (SwarmC2R) and stage-BC (fused
 * SwarmR2C + R2dbeC2R + quantize2bit) launch on the stream it runs on, and
 * around each one-launch wave of SDBE_STAGES_FUSED (fused_*).
 * sdbe_profile_read waits for the recorded events, returns the totals since
 * the last read and clears them.  launches counts every kernel sdbe_process
 * launched since the last read, enabled or not. */
typedef struct sdbe_profile {
    int64_t launches;
    int64_t stage_a_launches;
    int64_t stage_a_snapshots;   /* transforms done by those launches */
    double stage_a_ms;
    int64_t stage_bc_launches;
    int64_t stage_bc_chunks;
    double stage_bc_ms;
    int64_t fused_launches;      /* SDBE_STAGES_FUSED waves: one launch for stages A, B, C */
    int64_t fused_chunks;        /* chunks of those waves (snapshots = chunks * 143 / 128)  */
    double fused_ms;
    int64_t reserved[1];
} sdbe_profile;
int sdbe_profile_enable(sdbe_resampler *h, int32_t enable);
int sdbe_profile_read(sdbe_resampler *h, sdbe_profile *out);
/* Last error message of the handle (or of the thread for handle-less calls). */
int sdbe_last_error(const sdbe_resampler *h, char *buf, size_t n);

/* Pinned host buffers for packet groups and output groups.
 * Replace get_bgv_cpu_memory_cuda / get_vdg_cpu_memory_cuda
 * (vdif_in_databuf_cuda.cu:48-58, vdif_out_databuf_cuda.cu:48-58). */
int sdbe_host_alloc(void **ptr, size_t bytes);
int sdbe_host_free(void *ptr);

/* ---- stage entry points (device pointers), one per reference function ---- */
/* The kernels move data in 8- and 16-byte vectors, so device pointers must
 * be aligned (cudaMalloc and framework allocations are): 16 bytes for
 * packets, B-engine buffers, packed spectra, sdbe_swarm_c2r's output,
 * sdbe_resample_chunks' input and output and sdbe_quantize2bit's input;
 * 8 bytes for complex (c64) buffers and the float buffers of sdbe_swarm_r2c
 * and sdbe_r2dbe_c2r.  A misaligned pointer returns SDBE_ERR_ARG. */

/* vdif_to_beng (.cu:404-507) with its pre-zeroing memset (.cu:897-898):
 * int8 [n_frames][128][16384][2] (imag, real) per pol. */
int sdbe_vdif_to_beng(const void *packets, int64_t n_packets, uint64_t b_zero, int32_t n_frames,
                      int32_t channel_map, int8_t *beng0, int8_t *beng1, void *stream);

/* The packed form the fused path uses: per pol [snapshot][2048 u32], each
 * u32 = 8 channels x (2-bit real << 2 | 2-bit imag) nibbles, channel k of the
 * group in bits 4k..4k+3; missing packets filled with code 2 (value 0).
 * bitmap: [n_frames][256] bytes, bit f of byte c set per packet seen
 * (beng_frame_completion_t.cc, vdif_in_databuf.h:126-130); frame_counts:
 * [n_frames] int32; rejected: int32[1].  Arrays are accumulated into. */
int sdbe_unpack(const void *packets, int64_t n_packets, uint64_t b_zero, int32_t n_frames,
                int32_t channel_map, uint32_t *spec, int64_t pol_stride_words, int64_t snap0,
                uint32_t *bitmap, int32_t *frame_counts, int32_t *rejected, void *stream);
int sdbe_fill_missing(const uint32_t *bitmap, int32_t n_frames, int32_t channel_map, uint32_t *spec,
                      int64_t pol_stride_words, int64_t snap0, void *stream);

/* beng_int8_to_cufftComplex (.cu:532-556) + Nyquist zero (.cu:925-926):
 * int8 [n][16384][2] -> complex64 [n][16385]. */
int sdbe_beng_to_complex(const int8_t *beng, int64_t n_spectra, void *out_c64, void *stream);

/* SwarmC2R (.cu:589-625): packed spectra [n_snapshots][2048 u32] ->
 * float [n_snapshots][32768], unnormalised C2R.  This and
 * sdbe_resample_chunks compute in the handle's precision (SDBE_PRECISION_*). */
int sdbe_swarm_c2r(sdbe_resampler *h, const uint32_t *spec, int64_t n_snapshots, float *out,
                   void *stream);

/* SwarmR2C (.cu:631-667): float [n_chunks][36608] -> complex64 [n_chunks][18305]. */
int sdbe_swarm_r2c(sdbe_resampler *h, const float *in, int64_t n_chunks, void *out_c64, void *stream);

/* R2dbeC2R (.cu:673-709): complex64 [n_chunks][18305] from bin skip_chan ->
 * float [n_chunks][32768]. */
int sdbe_r2dbe_c2r(sdbe_resampler *h, const void *in_c64, int64_t n_chunks, int32_t skip_chan,
                   float *out, void *stream);

/* SwarmR2C and R2dbeC2R fused, chunk in -> resampled float chunk out. */
int sdbe_resample_chunks(sdbe_resampler *h, const float *in, int64_t n_chunks, float *out,
                         void *stream);

/* summary_stats + transform_reduce (.cu:66-137,953-977) in FP64:
 * out[0] = mean (quantizeOffset), out[1] = sqrt(M2/(n-1)) (quantizeThreshold).
 * The sums are of the samples minus the first one, so a large common offset
 * does not cancel digits of the variance.  Allocates n/256 (at most 1216)
 * pairs of FP64 partial sums on the stream and waits for it. */
int sdbe_summary_stats(const float *in, int64_t n, double *out_host, void *stream);

/* Allocation-free variant of sdbe_summary_stats.  No counterpart in the
 * reference.  For callers that cannot call cudaMalloc: a thread that shares
 * the device with asynchronous packet/payload copies (a cudaMalloc or
 * cudaFree can synchronize the whole device and stall them), or a process
 * held to a fixed, pre-reserved amount of device memory.  Its scratch is a fixed
 * 131,088-byte device array (8192 FP64 partial pairs + the result) that every
 * device loading the library holds until exit; n may be at most
 * SDBE_NOALLOC_MAX_SAMPLES (8192 partials x 16384 samples), larger n returns
 * SDBE_ERR_CAPACITY.  Each call looks up the array's address in the current
 * device's context, so calls after a cudaDeviceReset use the reloaded array.
 * Each call synchronizes its stream before returning (the result goes to host
 * memory), so no call can be made on a stream that is being captured into a
 * CUDA graph.  All calls share the array: calls that overlap on the GPU (other
 * streams, other host threads) race, so callers serialize them.  Nothing
 * accumulates in it across calls, so it needs no clearing.  Allocates
 * nothing, device or host. */
#define SDBE_NOALLOC_MAX_SAMPLES 134217728LL
int sdbe_summary_stats_noalloc(const float *in, int64_t n, double *out_host, void *stream);

/* quantize2bit (.cu:565-583): n floats -> n/16 words (n multiple of 16). */
int sdbe_quantize2bit(const float *in, uint32_t *out, int64_t n, float thresh, float offset,
                      void *stream);

/* Output VDIF headers (vdif_out_databuf.c:35-64 + vdif_out_net_thread.c:295-317)
 * for n_pkts frames of 8224 B per pol at frames + pol*pol_stride_bytes; packet
 * i gets df = (df0+i) mod 125000 with secs carried, psn = psn0+i. */
int sdbe_vdif_headers(void *frames, int64_t n_pkts, int64_t pol_stride_bytes, uint32_t secs0,
                      uint32_t df0, uint64_t psn0, uint32_t ref_epoch, uint32_t station_id,
                      uint32_t bdc_sideband, uint32_t rx_sideband, void *stream);

/* Inverse polyphase filter bank for PFB-mode spectra (Shaw's least-squares
 * inversion, software/prototyping/cuda/pfb_inverse.cu:213-488, with the
 * Hamming window of :51-53 over ntap*32768 samples): complex64
 * [nblock][16385] -> float [nblock+ntap-1][32768], the time blocks whose
 * forward PFB (pfb_inverse.cu:173-207) gives the spectra, minimum-norm where
 * the spectra leave them free.  Pseudo time stream by FP32 C2R, banded
 * P P^T solve and projection in FP64 (the systems are ill-conditioned).
 * 2 <= ntap <= 8; spec_c64 8-byte aligned.  The prototype compiles its
 * solve out (#if 0); this restates the method it sets up.  Uses handle
 * scratch of nblock*(4 + 8*ntap)*32768 bytes, allocated when a call needs
 * more than any earlier one (that growth synchronizes the device). */
int sdbe_inverse_pfb(sdbe_resampler *h, const void *spec_c64, int64_t nblock, int32_t ntap, float *out,
                     void *stream);

/* Mar-2015 snapshot reorder on packed spectra (prototyping/cuda/reorder.py:13-43):
 * [n_frames][128][2048 u32] -> [n_frames-1][128][2048 u32]. */
int sdbe_reorder_mar2015(const uint32_t *spec_in, int32_t n_frames, uint32_t *spec_out, void *stream);

/* ---- measurement helper (no counterpart in the reference) --------------- */
/* FP32 FMA rate of a device, TFLOP/s (2 flops per FMA), from one timed
 * launch of 16 independent FMA chains per thread, two 512-thread CTAs per
 * SM; *ms = the launch's CUDA-event time.  The roofline denominator of the
 * FP32 radix kernels, which are bound by FP32 issue. */
int sdbe_fp32_fma_rate(int32_t device, double *tflops, double *ms);

/* ---- test hook: bounded mbarrier waits (no counterpart in the reference) - */
/* Arms the next SDBE_PRECISION_TC16_FAST call of h to withhold one MMA
 * completion signal in its first inverse-transform launch and to bound every
 * mbarrier wait of that launch by limit_ns nanoseconds.  The wait that
 * depends on the withheld signal runs out; the kernel records the time-out
 * in h's status flag, stops waiting, frees its tensor memory and returns, so
 * the context stays usable.  The call after it returns SDBE_ERR_CUDA.  Used
 * by the tests of the failure path; limit_ns must be in [1e3, 1e9]. */
int sdbe_test_tc_timeout(sdbe_resampler *h, int64_t limit_ns);

/* ---- test hook: group assembly decisions (no counterpart in the reference) */
/* Copies to host memory the accept flag (1: inserted into a group) that the
 * device policy gave each packet of the last sdbe_ingest batch of h, in
 * arrival order (for 8pac input, of the 8 n unpacked packets).  n must equal
 * that batch's packet count.  Used by the tests of the group assembly. */
int sdbe_test_ingest_accept(const sdbe_resampler *h, uint8_t *mask, int64_t n);

#ifdef __cplusplus
}
#endif
#endif /* SDBE_H */
