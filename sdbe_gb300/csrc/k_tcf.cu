// The fast tensor-core form (SDBE_PRECISION_TC16_FAST): every transform runs
// as a chain of small DFT GEMMs on the 5th-generation tensor cores, with the
// twiddles and index permutations between them on the CUDA cores.
//
// Every GEMM stage is D[row][col] = sum_k X[row][k] G[col][k]: X holds the
// data as FP16 (re, im) pairs along K (the A operand, 128 rows per MMA), G
// the real form of the complex DFT matrix split into FP16 hi and lo halves,
// and D accumulates in FP32 in tensor memory: per K-step one MMA with the hi
// half and one with the lo half into the same accumulator, so the epilogue
// reads the compensated product directly.  The epilogue applies the
// twiddles in FP32 and rounds to FP16 into the next stage's operand: a
// transposition in which each thread's row scatters into the next stage's
// rows.  Row orders are chosen so that most scatters take one shared-memory
// wavefront per warp.  A whole stage's tiles accumulate side by side in
// tensor memory, so the MMAs of a stage issue back to back.
//
// Kernels (persistent over items):
//  * k_tcf_inv: a 16384-point inverse transform, radices 32 x 32 x 16 in
//    decimation in time (k = 512 n1 + 16 n2 + n3, m = k1 + 32 k2 + 1024 k3):
//      stage 1  rows n' = 16 n2 + n3 (512), DFT-32 over n1, twiddle W^(n' k1)
//      stage 2  rows (k1, n3)       (512), DFT-32 over n2, twiddle W_512^(n3 k2)
//      stage 3  rows (k1, k2)      (1024), DFT-16 over n3, output z[m].
//    Stage A's C2R 32768 per snapshot (input: the packed 2-bit spectrum) and
//    stage C's C2R 32768 per chunk (input: the R2C bins [skip, skip + 16384]
//    of stage B); the C2R pairing of the 16385 bins into 16384 complex values
//    is folded into the input step.  Two teams per CTA (an issuer warp and 8
//    epilogue warps each) take alternate items, each in its own operand
//    buffer and half of tensor memory, rewriting the operand in place stage
//    by stage; one team's CUDA-core steps overlap the other's MMAs.
//  * k_tcf_fwd: stage B's R2C 36608 per chunk, an 18304-point forward
//    transform of z[p] = x[2p] + i x[2p + 1] in the prime-factor map
//    18304 = 143 x 128 (143 = 11 x 13, 128 = 16 x 8): four stages DFT-16,
//    DFT-8, DFT-11, DFT-13 with one twiddle, W_128^(n8 k16), after the first;
//    then the R2C pairing and the trim to bins [skip, skip + 16384].  Warp 0
//    issues; warps 1-16 are four epilogue groups of four warps (one per
//    tensor-memory lane quarter); two operand buffers alternate by stage.
//
// MMAs are issued by an elected lane of a converged issuer warp.  Every
// mbarrier wait is bounded: on time-out the kernel records the failure in
// `status`, stops waiting and completes.
//
// Fixed power-of-two scales keep every FP16 operand below 2^16 in magnitude
// for any 2-bit input (per-stage bounds from the input energy: Parseval and
// Cauchy-Schwarz), and the outputs are scaled back exactly to cuFFT's
// unnormalised convention.
#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include <cmath>
#include <type_traits>
#include <cstring>
#include <vector>

#include "fft_core.cuh"
#include "handle.cuh"
#include "tcgen05.cuh"

namespace sdbe {
namespace {

using namespace tc5;

constexpr int kEpiWarps = 16;
constexpr int kEpiThreads = 32 * kEpiWarps;
constexpr int kThreads = 32 + kEpiThreads;
constexpr uint32_t kTmemCols = 512;

// Scales (powers of two, exact).  Stage A stores its time series x 2^-2
// (|x| <= 32768 * 2 sqrt 2 < 2^17).  Stage B scales by 2^-8 in its first
// twiddle: a stage of radix r multiplies the energy by r, a chunk's energy is
// at most 2 * 32768^2 * 8 before stage A's scale, so no value of its four
// stages exceeds 2^15 (Cauchy-Schwarz), and typical ones stay near 10 - 100.
// Its R2C bins carry a further 2^-1 (the C2R pairing's factor of two), and
// stage C scales its stages 1 and 2 by 2^-5 each.
constexpr float kScaleA = 0.25f;
constexpr float kScaleB = 1.f / 256.f;
constexpr float kScaleC1 = 1.f / 32.f, kScaleC2 = 1.f / 32.f;
// stage C output x 2^21 = back to the unnormalised value (2^-2 * 2^-8 * 2^-1 * 2^-10)
constexpr float kUnscaleC = 2097152.f, kRescaleC = 1.f / 2097152.f;

// ---- shared memory of k_tcf_inv (bytes from a 1024-byte aligned base) -----
constexpr uint32_t kOpBytes = 65536;                // one operand buffer (16384 complex FP16)
constexpr uint32_t kG32Bytes = 128 * 64 * 2;        // DFT-32, [hi | lo] x K 64
constexpr uint32_t kG16Bytes = 64 * 32 * 2;         // DFT-16, [hi | lo] x K 32
constexpr uint32_t kInvOffG = 2 * kOpBytes;
constexpr uint32_t kInvOffStg = kInvOffG + kG32Bytes + kG16Bytes;
// float2 tables: e^{2 pi i n1/64} (n1 <= 16, 32 slots), e^{2 pi i n'/32768} (512),
// e^{2 pi i n'/16384} (512, at n' + n'/16 so that 16 lanes with n' 16 apart
// hit distinct banks), e^{2 pi i n3/512} (16)
constexpr int kTabA1 = 0, kTabA2 = 32, kTabB = kTabA2 + 512, kTabC = kTabB + 544, kInvTabLen = kTabC + 16;
constexpr uint32_t kStgPacked = 2 * 8192, kStgBins = kTcfBinsLen * 4;  // packed: one snapshot per team
// packed input: two 16-entry float2 tables of a code pair's (e, d) parts, after the tables
constexpr uint32_t kPairLutBytes = 32 * 8;
constexpr uint32_t inv_smem(bool bins) {
    return kInvOffStg + (bins ? kStgBins : kStgPacked) + kInvTabLen * 8 + (bins ? 0u : kPairLutBytes) + 1024;
}

// ---- shared memory of k_tcf_fwd --------------------------------------------
constexpr uint32_t kFwdX0 = 90112;                  // raw chunk, DFT-8 operand, DFT-13 operand
constexpr uint32_t kFwdX1 = 80896;                  // DFT-16 operand, DFT-11 operand (+128-byte tail), Z
constexpr uint32_t kG16f = 64 * 32 * 2, kG8f = 32 * 16 * 2, kG11f = 64 * 32 * 2, kG13f = 64 * 32 * 2;
constexpr uint32_t kFwdOffG = kFwdX0 + kFwdX1;
constexpr uint32_t kFwdOffTab = kFwdOffG + kG16f + kG8f + kG11f + kG13f;
// float2 tables: 2^-8 W_128^(n8 k16) at 8 k16 + n8 (the 8 lanes of a row group read 8
// consecutive entries), W_36608^(128 a) (a <= 143, 144 slots), W_36608^b (b < 128)
constexpr int kTabW128 = 0, kTabQHi = 128, kTabQLo = kTabQHi + 144, kFwdTabLen = kTabQLo + 128;
constexpr uint32_t kFwdSmem = kFwdOffTab + kFwdTabLen * 8 + 1024;
static_assert(kFwdSmem <= 232448 && inv_smem(true) <= 232448, "shared memory above 227 KB");

// ---- device helpers --------------------------------------------------------
__device__ __forceinline__ void named_sync_epi() { asm volatile("bar.sync 1, %0;" ::"r"(kEpiThreads) : "memory"); }

__device__ __forceinline__ uint32_t sw32_off(int row, int kc) {
    return static_cast<uint32_t>((row >> 3) * 256 + (row & 7) * 32 + ((((kc >> 2) ^ ((row & 7) >> 2)) & 1) << 4) +
                                 (kc & 3) * 4);
}
// K-major, no swizzle, 3 core matrices (12 complex) per row group: the
// DFT-11 operand.  Its second K-step also reads a 4th core matrix, which is
// the next row group's first (finite data that meets zero columns of G).
__device__ __forceinline__ uint32_t k24_off(int row, int kc) {
    return static_cast<uint32_t>((row >> 3) * 384 + (kc >> 2) * 128 + (row & 7) * 16 + (kc & 3) * 4);
}

__device__ __forceinline__ float2 h2f(uint32_t w) {
    const __half2 h = *reinterpret_cast<const __half2 *>(&w);
    return __half22float2(h);
}

// Complex value i of 16 loaded accumulator columns (re, im pairs), i < 8.
__device__ __forceinline__ float2 acc2(const uint32_t *r, int i) {
    return make_float2(__uint_as_float(r[2 * i]), __uint_as_float(r[2 * i + 1]));
}

// Bulk copy global -> shared of `bytes` (multiple of 16), completing on mbar.
__device__ __forceinline__ void bulk_g2s(void *dst, const void *src, uint32_t bytes, uint64_t *mbar) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(mbar)), "r"(bytes)
                 : "memory");
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(smem_u32(dst)),
        "l"(src), "r"(bytes), "r"(smem_u32(mbar))
        : "memory");
}

// Bulk copy shared -> global of `bytes` (multiple of 16) in this thread's
// bulk group; the source may be rewritten after bulk_wait_read().
__device__ __forceinline__ void bulk_s2g(void *dst, const void *src, uint32_t bytes) {
    asm volatile("cp.async.bulk.global.shared::cta.bulk_group [%0], [%1], %2;" ::"l"(dst), "r"(smem_u32(src)),
                 "r"(bytes)
                 : "memory");
    asm volatile("cp.async.bulk.commit_group;" ::: "memory");
}
// Piece i (at most 16 KB) of an L2 prefetch of `bytes` (a multiple of 16) at
// the 16-byte aligned src; the calling threads take i = 0, 1, ... .
__device__ __forceinline__ void l2_prefetch_piece(const void *src, uint32_t bytes, int i) {
    const uint32_t off = 16384u * static_cast<uint32_t>(i);
    if (off < bytes) {
        const uint32_t n = bytes - off < 16384u ? bytes - off : 16384u;
        asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;" ::"l"(static_cast<const char *>(src) + off), "r"(n)
                     : "memory");
    }
}
__device__ __forceinline__ void bulk_wait_read() { asm volatile("cp.async.bulk.wait_group.read 0;" ::: "memory"); }
__device__ __forceinline__ void bulk_wait_all() { asm volatile("cp.async.bulk.wait_group 0;" ::: "memory"); }

// Common kernel state: barriers, tensor memory, error flag.
constexpr int kFull = 18;           // completion barriers, one per tile of a whole stage
struct Ctl {
    uint64_t full[kFull], ready[2], done, stg, b13;  // b13: an item's DFT-13 MMAs retired (chain)
    uint64_t lim;  // bound of every mbarrier wait (ns)
    int err;
};

__device__ __forceinline__ void ctl_init(Ctl &c, uint64_t lim) {
    c.lim = lim;
    for (int i = 0; i < kFull; ++i) mbar_init(&c.full[i], 1);
    mbar_init(&c.ready[0], kEpiWarps);
    mbar_init(&c.ready[1], kEpiWarps);
    mbar_init(&c.done, 1);
    mbar_init(&c.stg, 1);
    mbar_init(&c.b13, 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    c.err = 0;
}

__device__ __forceinline__ bool err_set(const Ctl &c) { return *reinterpret_cast<const volatile int *>(&c.err) != 0; }
__device__ __forceinline__ void raise_err(Ctl &c) { *reinterpret_cast<volatile int *>(&c.err) = 1; }

// MMA issuer state.  All of warp 0 runs the issuer (its values are warp
// uniform, so descriptors stay in uniform registers and cost no issue slots
// of the epilogue warps' pipes); one elected lane issues each MMA and commit.
struct Issuer {
    Ctl *c;
    uint32_t tb, rphase = 0;  // bit b: phase parity of ready[b]
    // One GEMM stage: every tile of the stage has its own accumulator
    // (tile j at column j * col_w) and completion barrier full[j], so the
    // stage issues without waiting; the epilogue's publish of the next
    // operand (after its last tensor-memory read) orders the next stage's
    // writes after this stage's reads.
    // With `mark` (an item's first stage), returns false without issuing when
    // the epilogue published the end mark (*mark < 0) instead of an operand.
    template <int KSTEPS>
    __device__ bool stage_all(int buf, uint32_t xa, int tiles, uint32_t tile_bytes, uint32_t kstep_bytes, uint32_t lbo,
                              uint32_t sbo, uint32_t layout, uint32_t g, uint32_t g_sbo, uint32_t g_lo, int n,
                              uint32_t col_w, const volatile int64_t *mark = nullptr) {
        asm volatile("" : "+r"(g), "+r"(xa));  // descriptors built here, not hoisted out of the item loop
        uint64_t gh[KSTEPS], gl[KSTEPS];
#pragma unroll
        for (int ks = 0; ks < KSTEPS; ++ks) {
            gh[ks] = desc(g + ks * 256, 128, g_sbo, kNoSwizzle);
            gl[ks] = desc(g + g_lo + ks * 256, 128, g_sbo, kNoSwizzle);
        }
        const uint64_t x0 = desc(xa, lbo, sbo, layout);
        const uint32_t id = idesc_f16(128, n);
        if (!err_set(*c) && !mbar_wait(&c->ready[buf], (rphase >> buf) & 1u, c->lim)) raise_err(*c);
        rphase ^= 1u << buf;
        __syncwarp();
        fence_after();
        if (mark && *mark < 0) return false;
        const bool ok = !err_set(*c);
        for (int j = 0; j < tiles; ++j) {
            if (ok) {
                const uint32_t d = tb + j * col_w;
                const uint64_t xj = x0 + ((j * tile_bytes) >> 4);
#pragma unroll
                for (int ks = 0; ks < KSTEPS; ++ks) {
                    const uint64_t xd = xj + ((ks * kstep_bytes) >> 4);
                    mma_f16_elect(d, xd, gh[ks], id, ks > 0);
                    mma_f16_elect(d, xd, gl[ks], id, true);
                }
            }
            commit_elect(&c->full[j]);
        }
        return true;
    }
    __device__ void finish() {  // every MMA retired before tensor memory is freed
        commit_elect(&c->done);
        if (!mbar_wait(&c->done, 0)) raise_err(*c);  // real completion of issued MMAs: the default bound
        __syncwarp();
    }
};

// Epilogue warp state of k_tcf_fwd: group grp (four warps, one per lane
// quarter) takes either its share of a stage's tiles (stage_group) or its
// share of every tile's columns (stage_all).
struct Epi {
    Ctl *c;
    int lane, grp, q, et;
    uint32_t tq;  // tensor-memory address of this warp's lane quarter, column 0
    uint32_t stg_uses = 0;
    __device__ void wait_staging() {
        if (!err_set(*c) && !mbar_wait(&c->stg, stg_uses & 1u, c->lim)) raise_err(*c);
        ++stg_uses;
    }
    // Phase parity of full[j] in bit j, flipped for every tile of a stage
    // when the stage is done (whether or not this warp waited on it).
    uint32_t fbits = 0;
    __device__ void wait_full(int j) {
        if (!err_set(*c) && !mbar_wait(&c->full[j], (fbits >> j) & 1u, c->lim)) raise_err(*c);
        fence_after();
    }
    // Runs f(j, accumulator address of tile j) on every tile of a whole stage.
    template <class F>
    __device__ void stage_all(int n, uint32_t col_w, F f) {
        for (int j = 0; j < n; ++j) {
            wait_full(j);
            f(j, tq + j * col_w);
        }
        fbits ^= (1u << n) - 1u;
    }
    // Runs f(j, ...) on the tiles j = grp + rot (mod 4) of a whole stage.
    template <class F>
    __device__ void stage_group(int n, uint32_t col_w, int rot, F f) {
        for (int j = (grp + rot) & 3; j < n; j += 4) {
            wait_full(j);
            f(j, tq + j * col_w);
        }
        fbits ^= (1u << n) - 1u;
    }
    // The next operand is written and this warp's tensor-memory reads are done.
    __device__ void publish_all(int buf) {
        fence_before();
        fence_async_smem();
        __syncwarp();
        if (lane == 0) mbar_arrive(&c->ready[buf]);
    }
};

template <class A>
__device__ __forceinline__ int seg_index(const A &a, int64_t item) {
    int j = 0;
    while (j + 1 < a.n && item >= a.s[j + 1].item0) ++j;
    return j;
}


// Item order and cross-stage dependencies of a persistent stage loop.  Static
// (ticket null): CTA b takes items b, b + G, b + 2G, ... (G CTAs).  Chain (one
// launch runs stages A, B and C of a wave, k_tcf_chain): items are tickets
// from a global counter, handed out in order to running CTAs, and a CTA takes
// the next stage's tickets only once the current stage's run out, so every
// item a later stage waits for is already held by a running CTA; each wait is
// bounded.
struct Sched {
    unsigned *ticket;      // null: static order
    const unsigned *dep;   // counters the items wait for (stage B: per stage-A batch; stage C: per stage-B item)
    unsigned *done;        // counters the items bump once their output is in global memory
};

// Bounded wait (global time) until *p >= want, with acquire ordering.
__device__ __forceinline__ bool wait_count(const unsigned *p, unsigned want, uint64_t limit_ns) {
    unsigned v;
    asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    if (v >= want) return true;
    const uint64_t t0 = global_ns();
    for (;;) {
        __nanosleep(256);
        asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
        if (v >= want) return true;
        if (global_ns() - t0 > limit_ns) return false;
    }
}
// A counter bump after this thread's (or, behind a barrier, its CTA's) global
// writes, with release ordering: a wait_count that sees it sees the writes.
__device__ __forceinline__ void bump(unsigned *p) {
    asm volatile("red.release.gpu.global.add.u32 [%0], 1;" ::"l"(p) : "memory");
}
// Generic-proxy accesses ordered with this thread's bulk (async-proxy) copies of global memory.
__device__ __forceinline__ void fence_proxy_global() { asm volatile("fence.proxy.async.global;" ::: "memory"); }

__device__ __forceinline__ void tmem_alloc_cols(uint32_t *dst) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(dst)),
                 "r"(kTmemCols));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
}
__device__ __forceinline__ void tmem_free_cols(uint32_t base) {
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(base), "r"(kTmemCols));
}

// Shared item slots of a chain phase: [t] team t's current item, its issuer's
// mark (< 0: end), [2 + 4 t + 2 p ..] team t's (item, next) pair p, [10 + s %
// 4] the item of stage C's staging fill s, [14 + k % 2] stage B's k-th item,
// [18 + t] team t's item whose stage-A series awaits its completion signal.
// The team leaders keep this state here rather than in registers: the stage-A
// loop body runs at the register cap.
constexpr int kSlots = 20;

// ============================================================================
// k_tcf_inv: 16384-point inverse transforms (stages A and C)
// ============================================================================
enum : int { IN_PACKED = 0, IN_BINS = 1 };
enum : int { OUT_TS_HALF = 0, OUT_TS_FLOAT = 1, OUT_QUANT = 2, OUT_FLOAT_MOMENTS = 3, OUT_QUANT_SUMS = 4, OUT_FLOAT = 5 };

struct SegInv {
    const void *in;          // packed spectra (u32 words) or R2C bins (half2, kTcfBinsLen per chunk)
    void *out;               // stage A: time series [pol][n][32768], half or float
    int64_t in_pol_stride;   // words (packed) or bins
    int64_t first, n;        // first snapshot (packed input), items per pol
    int64_t out_pol_stride;  // elements
    int64_t item0;
    ResampleOut o;           // stage C: payload target, thresholds, floats, partials
};
struct ArgsInv {
    int64_t n_items;
    int n;
    SegInv s[kMaxSegs];
    const uint8_t *g;        // inverse DFT-32 then DFT-16 matrices, pre-tiled
    const float2 *tab;       // the kInvTabLen twiddle values
    int *status;             // set to 1 on a barrier time-out (host-mapped)
    uint64_t wait_ns;        // bound of every mbarrier wait
    int withhold;            // 1: team 0 withholds its first stage commit (test of the time-out path)
};

// Staged packed spectrum: word w at w ^ ((w >> 6) & 1) ^ (((w >> 7) & 1) << 4),
// so that the input step's 32 lanes (8 values of n2 % 8 x 4 of n1 % 4) read
// 32 distinct banks.
__device__ __forceinline__ uint32_t stg_pos(uint32_t w) { return w ^ ((w >> 6) & 1u) ^ (((w >> 7) & 1u) << 4); }

__device__ __forceinline__ float2 stg_value(const uint32_t *stg, int k) {
    const uint32_t w = stg[stg_pos(static_cast<uint32_t>(k) >> 3)] >> ((k & 7) * 4);
    const float re = __uint_as_float(0x4B400000u | ((w >> 2) & 3u)) - 12582914.0f;
    const float im = __uint_as_float(0x4B400000u | (w & 3u)) - 12582914.0f;
    return make_float2(re, im);
}

// Two teams per CTA, each of one MMA-issuer warp and 8 epilogue warps (two
// per tensor-memory lane quarter), work on alternate items: team t owns
// operand buffer t, tensor-memory columns [256 t, 256 t + 256) and its own
// barriers, so one team's CUDA-core steps run while the other's MMAs do.
// Within a team a stage's four or eight tiles accumulate side by side in its
// 256 columns, one commit per stage, and the epilogue rewrites the operand
// buffer in place once the stage's MMAs have all completed.
constexpr int kTeamEpiWarps = 8, kTeamEpiThreads = 32 * kTeamEpiWarps;
constexpr int kInvThreads = 2 * (32 + kTeamEpiThreads);
constexpr uint32_t kStgTeam = kStgPacked / 2;  // packed staging per team (bytes)
static_assert(kStgPacked == 2 * 8192, "packed staging: one 8 KB snapshot per team");

struct CtlInv {
    uint64_t ready[2], mma[2], stg[2], done[2];
    int err;
};

// The kernels' control state in static shared memory: the inverse phases'
// barriers (two sets, for stages A and C of a chain), the forward phase's,
// the teams' FP64 partial sums, the item slots and the tensor-memory base.
__shared__ __align__(8) CtlInv g_ctl_inv[2];
__shared__ __align__(8) Ctl g_ctl_fwd;
__shared__ double g_red[2][2 * kTeamEpiWarps];
__shared__ int64_t g_slots[kSlots];
__shared__ uint32_t g_tmem_base;

// One stage-A or stage-C loop over its items (a whole k_tcf_inv launch, or a
// phase of k_tcf_chain): sm is the 1024-byte aligned dynamic shared memory,
// tmem_base the CTA's 512 tensor-memory columns.  Ends with a CTA barrier,
// every MMA retired and every bulk store complete.
template <int IN, int OUT, int CI, bool CHAIN>
__device__ __forceinline__ void inv_phase(const ArgsInv &a, const Sched sc, uint8_t *sm, uint32_t tmem_base) {
    CtlInv &ctl = g_ctl_inv[CI];
    auto &red = g_red;
    volatile int64_t *slots = g_slots;
    constexpr bool kBins = IN == IN_BINS;
    constexpr bool kQuant = OUT == OUT_QUANT || OUT == OUT_QUANT_SUMS;  // 2-bit payload out, bulk-stored
    uint32_t *stg_all = reinterpret_cast<uint32_t *>(sm + kInvOffStg);
    float2 *tab = reinterpret_cast<float2 *>(sm + kInvOffStg + (kBins ? kStgBins : kStgPacked));
    // C2R pairing of two 2-bit code nibbles y and ym (re code at bits 2-3, im
    // code at bits 0-1): (e, d) = (y + conj ym, y - conj ym), exact small
    // integers, as two tables of 16 entries (128 bytes each, so a half-warp's
    // loads hit distinct banks or broadcast): entry (yr << 2 | mr) holds
    // (Re e, Re d) = (yr + mr, yr - mr), entry 16 + (yi << 2 | mi) holds
    // (Im e, Im d) = (yi - mi, yi + mi)
    float2 *pair_lut = tab + kInvTabLen;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int t = warp >= 9 ? 1 : 0;          // team
    const int tw = warp - 9 * t;              // warp within the team: 0 issuer, 1-8 epilogue
    uint8_t *const X = sm + t * kOpBytes;     // this team's operand

    if (tid == 0) {
        for (int i = 0; i < 2; ++i) {
            mbar_init(&ctl.ready[i], kTeamEpiWarps);
            mbar_init(&ctl.mma[i], 1);
            mbar_init(&ctl.stg[i], 1);
            mbar_init(&ctl.done[i], 1);
        }
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        ctl.err = 0;
    }
    {
        const uint4 *src = reinterpret_cast<const uint4 *>(a.g);
        uint4 *dst = reinterpret_cast<uint4 *>(sm + kInvOffG);
        for (int i = tid; i < static_cast<int>((kG32Bytes + kG16Bytes) / 16); i += kInvThreads) dst[i] = __ldg(src + i);
        for (int i = tid; i < kInvTabLen; i += kInvThreads) tab[i] = __ldg(a.tab + i);
        if (!kBins && tid < 32) {
            const float y = static_cast<float>((tid >> 2) & 3) - 2.f, m = static_cast<float>(tid & 3) - 2.f;
            pair_lut[tid] = tid < 16 ? make_float2(y + m, y - m) : make_float2(y - m, y + m);
        }
    }
    fence_async_smem();
    fence_before();
    __syncthreads();
    fence_after();
    const uint32_t tb = tmem_base + 256u * t;
    auto err_on = [&]() { return *reinterpret_cast<const volatile int *>(&ctl.err) != 0; };
    auto raise = [&]() { *reinterpret_cast<volatile int *>(&ctl.err) = 1; };
    auto item_of = [&](int64_t m) { return static_cast<int64_t>(blockIdx.x) + m * gridDim.x; };
    const uint64_t lim = a.wait_ns;

    auto item_in = [&](int64_t item) -> const void * {
        const SegInv &s = a.s[seg_index(a, item)];
        const int64_t local = item - s.item0;
        const int64_t pol = local >= s.n ? 1 : 0, loc = local - pol * s.n;
        if constexpr (kBins)
            return static_cast<const uint32_t *>(s.in) +
                   (pol * s.in_pol_stride + loc * static_cast<int64_t>(kTcfBinsLen));
        else
            return static_cast<const uint32_t *>(s.in) + pol * s.in_pol_stride + (s.first + loc) * kGroups;
    };
    // Chain, stage C: the bins staging is filled in the CTA's fill sequence
    // by the MMA issuer of the team that has read the fill before (fill s + 1
    // once team s % 2 has published its stage-1 operand).  A fill takes a
    // ticket, waits for that item's bins, records the item in slot 10 + s % 4
    // and copies; without an item it ends both teams (fills s and s + 1 marked
    // -1, both staging barriers released).
    auto fill_stg = [&](int64_t fs) {
        int64_t z = static_cast<int64_t>(atomicAdd(sc.ticket, 1u));
        if (z >= a.n_items) z = -1;
        slots[10 + (fs & 3)] = z;
        if (z < 0) {
            slots[10 + ((fs + 1) & 3)] = -1;
            mbar_arrive(&ctl.stg[fs & 1]);
            mbar_arrive(&ctl.stg[(fs + 1) & 1]);
            return;
        }
        if (!err_on() && !wait_count(sc.dep + z, 1u, lim)) raise();
        fence_proxy_global();
        fence_async_smem();
        bulk_g2s(stg_all, item_in(z), kStgBins, &ctl.stg[fs & 1]);
    };

    if (tw == 0) {
        // ---- MMA issuer of team t (whole warp; an elected lane issues) ----
        const uint32_t g32 = smem_u32(sm + kInvOffG), g16 = g32 + kG32Bytes;
        uint32_t rph = 0;
        bool withhold = a.withhold != 0 && t == 0;
        // One GEMM stage; the first of an item returns false at the end mark.
        auto stage = [&](auto ksteps_c, int tiles, uint32_t tile_bytes, uint32_t lbo, uint32_t sbo, uint32_t layout,
                         uint32_t g, uint32_t g_sbo, uint32_t g_lo, int n, uint32_t col_w, bool first) -> bool {
            constexpr int KSTEPS = decltype(ksteps_c)::value;
            uint32_t xa = smem_u32(X);
            asm volatile("" : "+r"(g), "+r"(xa));  // descriptors built here, not hoisted out of the item loop
            uint64_t gh[KSTEPS], gl[KSTEPS];
#pragma unroll
            for (int ks = 0; ks < KSTEPS; ++ks) {
                gh[ks] = desc(g + ks * 256, 128, g_sbo, kNoSwizzle);
                gl[ks] = desc(g + g_lo + ks * 256, 128, g_sbo, kNoSwizzle);
            }
            const uint64_t x0 = desc(xa, lbo, sbo, layout);
            const uint32_t id = idesc_f16(128, n);
            if (!err_on() && !mbar_wait(&ctl.ready[t], rph, lim)) raise();
            rph ^= 1u;
            __syncwarp();
            fence_after();
            if (first && slots[t] < 0) return false;  // the team has no more items
            if (!err_on()) {
                for (int j = 0; j < tiles; ++j) {
                    const uint64_t xj = x0 + ((j * tile_bytes) >> 4);
#pragma unroll
                    for (int ks = 0; ks < KSTEPS; ++ks) {
                        const uint64_t xd = xj + ((ks * 32) >> 4);
                        mma_f16_elect(tb + j * col_w, xd, gh[ks], id, ks > 0);
                        mma_f16_elect(tb + j * col_w, xd, gl[ks], id, true);
                    }
                }
            }
            if (withhold)
                withhold = false;  // test of the time-out path: this stage's completion is never signalled
            else
                commit_elect(&ctl.mma[t]);
            return true;
        };
        if constexpr (CHAIN) {
            // the team's items until its epilogue publishes the end mark; in
            // stage C the issuer also makes the fill after the team's (in its
            // idle time, after the stage-1 MMAs are issued)
            int64_t fs = t;
            if (kBins && t == 0 && lane == 0) fill_stg(0);
            __syncwarp();
            while (stage(std::integral_constant<int, 4>{}, 4, 16384, 16, 1024, kSwizzle128, g32, 1024, 8192, 64, 64,
                         true)) {
                if (kBins && lane == 0) fill_stg(fs + 1);
                __syncwarp();
                fs += 2;
                stage(std::integral_constant<int, 4>{}, 4, 16384, 16, 1024, kSwizzle128, g32, 1024, 8192, 64, 64, false);
                stage(std::integral_constant<int, 2>{}, 8, 8192, 16, 512, kSwizzle64, g16, 512, 2048, 32, 32, false);
            }
        } else {
            for (int64_t m = t; item_of(m) < a.n_items; m += 2) {
                stage(std::integral_constant<int, 4>{}, 4, 16384, 16, 1024, kSwizzle128, g32, 1024, 8192, 64, 64, false);
                stage(std::integral_constant<int, 4>{}, 4, 16384, 16, 1024, kSwizzle128, g32, 1024, 8192, 64, 64, false);
                stage(std::integral_constant<int, 2>{}, 8, 8192, 16, 512, kSwizzle64, g16, 512, 2048, 32, 32, false);
            }
        }
        commit_elect(&ctl.done[t]);  // every MMA of the team retired before tensor memory is freed
        if (!mbar_wait(&ctl.done[t], 0)) raise();  // real completion of issued MMAs: the default bound
        __syncwarp();
    } else {
        // ---- epilogue warps of team t ----------------------------------------
        const int e = tw - 1;                       // 0..7
        const int q = warp & 3, h = e >> 2;         // lane quarter, which of its two warps
        const int et = e * 32 + lane;               // 0..255
        const uint32_t tq = tb + (static_cast<uint32_t>(q * 32) << 16);
        uint32_t mph = 0, sph = 0;
        uint32_t *stg = kBins ? stg_all : stg_all + t * (kStgTeam / 4);
        auto team_sync = [&]() { asm volatile("bar.sync %0, %1;" ::"r"(1 + t), "r"(kTeamEpiThreads) : "memory"); };
        auto wait_mma = [&]() {
            if (!err_on() && !mbar_wait(&ctl.mma[t], mph, lim)) raise();
            mph ^= 1u;
            fence_after();
        };
        auto publish = [&]() {  // this warp's part of the operand written, its tensor-memory reads done
            fence_before();
            fence_async_smem();
            __syncwarp();
            if (lane == 0) mbar_arrive(&ctl.ready[t]);
        };
        // packed input: each thread holds 32 bytes of the team's next snapshot
        uint4 pre0 = make_uint4(0, 0, 0, 0), pre1 = pre0;
        auto prefetch = [&](int64_t z) {
            const uint4 *src = reinterpret_cast<const uint4 *>(item_in(z));
            pre0 = __ldg(src + 2 * et);
            pre1 = __ldg(src + 2 * et + 1);
        };
        // chain: a stage-A ticket of this team, -1 at the end
        auto ticket_a = [&]() -> int64_t {
            const int64_t z = static_cast<int64_t>(atomicAdd(sc.ticket, 1u));
            return z < a.n_items ? z : -1;
        };
        auto land = [&]() {  // staged word w at stg_pos(w)
#pragma unroll
            for (int i = 0; i < 2; ++i) {
                const uint4 p = i ? pre1 : pre0;
                const uint32_t w = 8u * static_cast<uint32_t>(et) + 4u * i;
                const uint32_t u0 = (w >> 6) & 1u, u1 = (w >> 7) & 1u;
                const uint4 v = u0 ? make_uint4(p.y, p.x, p.w, p.z) : p;
                *reinterpret_cast<uint4 *>(stg + (w ^ (u1 << 4))) = v;
            }
        };
        auto nib = [](uint32_t w) {  // low nibble of w -> (real code - 2, imag code - 2)
            const float re = __uint_as_float(0x4B400000u | ((w >> 2) & 3u)) - 12582914.0f;
            const float im = __uint_as_float(0x4B400000u | (w & 3u)) - 12582914.0f;
            return make_float2(re, im);
        };

        // ---- input step: C2R pairing into the stage-1 operand -------------------
        // Packed input (stage A): row n' = 16 n2 + n3 at 32 n3 + n2; a warp takes
        // n3 = e and 15 - e, (n2 % 8, n1 % 4) = its lane, so that its 16 pairs k =
        // 512 (4 A + u) + 16 (8 B + a) + n3 (A, B < 4) have staging positions,
        // shifts and store offsets that are per-lane constants plus compile-time
        // ones.  Bins input (stage C): rows in natural order n'; a thread takes
        // n' = et and et + 256, four consecutive n1 per 16-byte store.
        auto input_n3 = [&](int n3, auto may_be_0) {  // may_be_0: std::bool_constant, n3 = 0 possible
            const int av = lane & 7, u = lane >> 3;
            float2 tB[4];  // W_32768^n', n' = 16 (8 B + av) + n3
#pragma unroll
            for (int i = 0; i < 4; ++i) tB[i] = tab[kTabA2 + 16 * (8 * i + av) + n3];
            if (!decltype(may_be_0)::value || n3 != 0) {
                const int u0 = u & 1, u1 = u >> 1;
                const int wl = 64 * u + 2 * av + ((n3 >> 3) ^ u0);
                const int L0 = wl + 16 * u1, L1 = wl + 16 * (1 - u1);
                const int sh = (n3 & 7) * 4, shm = ((8 - (n3 & 7)) & 7) * 4;
                uint8_t *S = X + 4096 * n3 + 128 * av + 4 * u;
                uint8_t *Sm = X + 4096 * (16 - n3) + 128 * (31 - av) + 12 - 4 * u;
#pragma unroll
                for (int it = 0; it < 16; ++it) {
                    const int A = it >> 2, B = it & 3;
                    const float2 tA = tab[kTabA1 + 4 * A + u];
                    const int xA = 16 * (A ^ av);
                    const int pos = 256 * A + 32 * (B >> 1) + ((B & 1) ? L1 : L0);
                    float2 zk, zm;
                    if (n3 != 8) {
                        const uint32_t yn = stg[pos] >> sh, mn = stg[pos ^ 2030] >> shm;
                        const float2 lr = pair_lut[(yn & 12u) | ((mn >> 2) & 3u)];
                        const float2 li = pair_lut[16u | ((yn << 2) & 12u) | (mn & 3u)];
                        const float2 tt = cmul(make_float2(lr.y, li.y), cmul(tA, tB[B]));
                        zk = make_float2(lr.x - tt.y, li.x + tt.x);
                        zm = make_float2(lr.x + tt.y, tt.x - li.x);
                    } else {  // k % 8 = 0: the mirror's word is 2048 - w
                        const int k = 512 * (4 * A + u) + 16 * (8 * B + av) + 8;
                        c2r_pair(nib(stg[pos] >> sh), stg_value(stg, kMA - k), cmul(tA, tB[B]), zk, zm);
                    }
                    *reinterpret_cast<uint32_t *>(S + 1024 * B + xA) = pack_half2(zk.x, zk.y);
                    *reinterpret_cast<uint32_t *>(Sm - 1024 * B + xA) = pack_half2(zm.x, zm.y);
                }
            } else {
                // n3 = 0: k = 512 n1 + 16 n2 is nibble 0 of word w = k / 8, and its
                // mirror 16384 - k (word 2048 - w) lies in the same row group, at
                // (31 - n1, 32 - n2) for n2 > 0 and at (32 - n1, 0) for n2 = 0.
                // k = 0 (lane 0, first pair) drops Im X[0] and pairs with the zero
                // bin 16384; k = 8192, its own mirror, follows the loop.
#pragma unroll 2
                for (int it = 0; it < 16; ++it) {
                    const int A = it >> 2, B = it & 3;
                    const int n1 = 4 * A + u, n2 = 8 * B + av;
                    const uint32_t w = static_cast<uint32_t>(64 * n1 + 2 * n2);
                    float2 y = nib(stg[stg_pos(w)]);
                    float2 ym = nib(stg[stg_pos((2048u - w) & 2047u)]);
                    const bool dc = it == 0 && lane == 0;
                    if (dc) {
                        y.y = 0.f;
                        ym = make_float2(0.f, 0.f);
                    }
                    float2 zk, zm;
                    c2r_pair(y, ym, cmul(tab[kTabA1 + n1], tab[kTabA2 + 16 * n2]), zk, zm);
                    *reinterpret_cast<uint32_t *>(X + sw128_off(n2, n1)) = pack_half2(zk.x, zk.y);
                    const bool n2z = B == 0 && av == 0;
                    if (!dc)
                        *reinterpret_cast<uint32_t *>(X + sw128_off(n2z ? 0 : 32 - n2, n2z ? 32 - n1 : 31 - n1)) =
                            pack_half2(zm.x, zm.y);
                }
                if (lane == 0) {  // k = 8192, its own mirror
                    const float2 y = stg_value(stg, kMA / 2);
                    float2 zk, zm;
                    c2r_pair(y, y, cmul(tab[kTabA1 + 16], tab[kTabA2]), zk, zm);
                    *reinterpret_cast<uint32_t *>(X + sw128_off(0, 16)) = pack_half2(zk.x, zk.y);
                }
            }
        };
        auto input_row = [&](int np) {
            const float2 wb = tab[kTabA2 + np];
#pragma unroll 1
            for (int c = 0; c < 4; ++c) {
                uint32_t zk[4], zm[4];
#pragma unroll
                for (int i = 0; i < 4; ++i) {
                    const int n1 = 4 * c + i, k = 512 * n1 + np;
                    float2 y = h2f(stg[k]), ym = h2f(stg[kMA - k]);
                    if (k == 0) {  // Im of bins 0 and 16384 are ignored (C2R)
                        y.y = 0.f;
                        ym.y = 0.f;
                    }
                    float2 a0, a1;
                    c2r_pair(y, ym, cmul(tab[kTabA1 + n1], wb), a0, a1);
                    zk[i] = pack_half2(a0.x, a0.y);
                    zm[i] = pack_half2(a1.x, a1.y);
                }
                *reinterpret_cast<uint4 *>(X + sw128_off(np, 4 * c)) = make_uint4(zk[0], zk[1], zk[2], zk[3]);
                if (np != 0) {  // mirrors 16384 - k: row 512 - n', K 31 - n1 (a 4-aligned group, reversed)
                    *reinterpret_cast<uint4 *>(X + sw128_off(512 - np, 28 - 4 * c)) =
                        make_uint4(zm[3], zm[2], zm[1], zm[0]);
                } else {  // row 0: 16384 - 512 n1 lies at K 32 - n1; n1 = 0 mirrors the Nyquist bin
#pragma unroll
                    for (int i = 0; i < 4; ++i)
                        if (4 * c + i > 0) *reinterpret_cast<uint32_t *>(X + sw128_off(0, 32 - 4 * c - i)) = zm[i];
                }
            }
            if (np == 0) {  // k = 8192, its own mirror
                const float2 y = h2f(stg[kMA / 2]);
                float2 zk, zm;
                c2r_pair(y, y, cmul(tab[kTabA1 + 16], tab[kTabA2]), zk, zm);
                *reinterpret_cast<uint32_t *>(X + sw128_off(0, 16)) = pack_half2(zk.x, zk.y);
            }
        };

        // The 32 DFT outputs of this thread's row (tile at tensor-memory address
        // t), times w0 b^k: two interleaved twiddle chains (steps b^2); output k
        // goes to d0 + 2048 k.
        auto twiddled32 = [&](uint32_t taddr, float2 b, float2 w0, uint8_t *d0) {
            const float2 b2 = cmul(b, b);
            float2 wa = w0, wb = cmul(w0, b);
#pragma unroll
            for (int hf = 0; hf < 2; ++hf) {
                uint32_t r0[16], r1[16];
                tmem_ld16(taddr + 32 * hf, r0);
                tmem_ld16(taddr + 32 * hf + 16, r1);
                tmem_wait<16>(r0, r1);
#pragma unroll
                for (int i = 0; i < 16; i += 2) {
                    const float2 y0 = cmul(acc2(i < 8 ? r0 : r1, i & 7), wa);
                    const float2 y1 = cmul(acc2(i < 8 ? r0 : r1, (i & 7) + 1), wb);
                    wa = cmul(wa, b2);
                    wb = cmul(wb, b2);
                    *reinterpret_cast<uint32_t *>(d0 + 2048 * (16 * hf + i)) = pack_half2(y0.x, y0.y);
                    *reinterpret_cast<uint32_t *>(d0 + 2048 * (16 * hf + i + 1)) = pack_half2(y1.x, y1.y);
                }
            }
        };
        // ---- stage 1 -> stage-2 operand (in place): row 16 k1 + n3, K n2, at
        // 2048 k1 + (offset of row n3, K n2) in the 128-byte swizzle
        auto epi1 = [&](int j) {
            int n2, n3;
            if constexpr (!kBins) {  // row n' = 16 lane + n3, n3 = 4 j + q
                n3 = 4 * j + q;
                n2 = lane;
            } else {                 // natural rows: n' = 128 j + 32 q + lane
                const int np = 128 * j + 32 * q + lane;
                n3 = np & 15;
                n2 = np >> 4;
            }
            const int np = 16 * n2 + n3;
            twiddled32(tq + 64 * j, tab[kTabB + np + (np >> 4)], make_float2(kBins ? kScaleC1 : 1.f, 0.f),
                       X + sw128_off(n3, n2));
        };
        // ---- stage 2 -> stage-3 operand (in place): row 32 k2 + k1, K n3, at
        // 2048 k2 + (offset of row k1, K n3) in the 64-byte swizzle
        auto epi2 = [&](int j) {
            const int r = 128 * j + 32 * q + lane, k1 = r >> 4, n3 = r & 15;
            // stage A's FP16 time series is a quarter of the unnormalised value
            twiddled32(tq + 64 * j, tab[kTabC + n3],
                       make_float2(kBins ? kScaleC2 : (OUT == OUT_TS_HALF ? kScaleA : 1.f), 0.f), X + sw64_off(k1, n3));
        };
        // ---- stage 3 -> output.  Row 32 k2 + k1 = 128 j + 32 q + lane, column k3:
        // z[m], m = k1 + 32 k2 + 1024 k3, = samples (2m, 2m + 1); a warp covers 32
        // consecutive m.
        float f1 = 0.f, f2 = 0.f;  // OUT_QUANT_SUMS: this thread's sums over the chunk (scaled values)
        double d1 = 0.0, d2 = 0.0; // OUT_FLOAT_MOMENTS
        auto epi3 = [&](int j, const SegInv &s, int64_t pol, int64_t loc) {
            const int r = 128 * j + 32 * q + lane;
            uint32_t r0[16], r1[16];
            tmem_ld16(tq + 32 * j, r0);
            tmem_ld16(tq + 32 * j + 16, r1);
            tmem_wait<16>(r0, r1);
            float2 v[16];
#pragma unroll
            for (int i = 0; i < 16; ++i) v[i] = acc2(i < 8 ? r0 : r1, i & 7);
            if constexpr (OUT == OUT_TS_HALF) {  // into the operand buffer, then one bulk store
#pragma unroll
                for (int i = 0; i < 16; ++i)
                    reinterpret_cast<uint32_t *>(X)[r + 1024 * i] = pack_half2(v[i].x, v[i].y);
            } else if constexpr (OUT == OUT_TS_FLOAT) {
                const int64_t off = pol * s.out_pol_stride + loc * static_cast<int64_t>(kNA);
#pragma unroll
                for (int i = 0; i < 16; ++i)
                    __stcs(reinterpret_cast<float2 *>(static_cast<float *>(s.out) + off) + r + 1024 * i, v[i]);
            } else if constexpr (OUT == OUT_FLOAT || OUT == OUT_FLOAT_MOMENTS) {
                float2 *fo = reinterpret_cast<float2 *>(s.o.fout + pol * s.o.fout_pol_stride + loc * kNC);
#pragma unroll
                for (int i = 0; i < 16; ++i) {
                    const float2 x = make_float2(kUnscaleC * v[i].x, kUnscaleC * v[i].y);
                    __stcs(fo + r + 1024 * i, x);
                    if constexpr (OUT == OUT_FLOAT_MOMENTS) {
                        d1 += static_cast<double>(x.x) + static_cast<double>(x.y);
                        d2 += static_cast<double>(x.x) * x.x + static_cast<double>(x.y) * x.y;
                    }
                }
            } else {
                // 2-bit codes against thresholds scaled like the values (powers
                // of two: the same codes as on the unscaled values).  Word
                // (r >> 3) + 128 k3 holds outputs r' + 1024 k3 of the 8 lanes
                // r' = r & ~7 .. + 7 (lane c at bits 4c); each lane builds its
                // codes of k3 < 8 and k3 >= 8 as two words (k3 at bits 4 (k3 % 8)),
                // an 8 x 8 nibble transpose over the 8 lanes leaves lane c with
                // the words of k3 = c and 8 + c.
                // the chunk's 8192-byte payload is staged in the (consumed) operand
                // buffer and leaves in one bulk store after the stage
                uint32_t *words = reinterpret_cast<uint32_t *>(X);
                const float th = kRescaleC * s.o.thr[pol], off = kRescaleC * s.o.thr[2 + pol];
                uint32_t wl = 0, wh = 0;
#pragma unroll
                for (int i = 0; i < 8; ++i) {
                    wl |= (code2(v[i].x, th, off) | (code2(v[i].y, th, off) << 2)) << (4 * i);
                    wh |= (code2(v[8 + i].x, th, off) | (code2(v[8 + i].y, th, off) << 2)) << (4 * i);
                }
                if constexpr (OUT == OUT_QUANT_SUMS) {
#pragma unroll
                    for (int i = 0; i < 16; ++i) {
                        f1 += v[i].x + v[i].y;
                        f2 = fmaf(v[i].x, v[i].x, fmaf(v[i].y, v[i].y, f2));
                    }
                }
                const int c = lane & 7;
                wl = nib_transpose8(wl, c);
                wh = nib_transpose8(wh, c);
                words[(r >> 3) + 128 * c] = wl;
                words[(r >> 3) + 128 * (8 + c)] = wh;
            }
        };
        // Per-chunk statistics of stage C (the team's 8 warps, after stage 3).
        auto chunk_stats = [&](const SegInv &s, int64_t pol, int64_t loc) {
            if constexpr (OUT == OUT_FLOAT_MOMENTS || OUT == OUT_QUANT_SUMS) {
                if (s.o.partials == nullptr) return;
                double s1, s2;
                if constexpr (OUT == OUT_FLOAT_MOMENTS) {
                    s1 = warp_sum(d1);
                    s2 = warp_sum(d2);
                } else {  // sums of the scaled values: x 2^21 and x 2^42 (exact)
                    s1 = static_cast<double>(warp_sum_f(f1)) * kUnscaleC;
                    s2 = static_cast<double>(warp_sum_f(f2)) * kUnscaleC * kUnscaleC;
                }
                if (lane == 0) {
                    red[t][e] = s1;
                    red[t][kTeamEpiWarps + e] = s2;
                }
                team_sync();
                if (et == 0) {
                    double t1 = 0.0, t2 = 0.0;
                    for (int w = 0; w < kTeamEpiWarps; ++w) {
                        t1 += red[t][w];
                        t2 += red[t][kTeamEpiWarps + w];
                    }
                    double *pp = s.o.partials + (pol * s.n + loc) * 3;
                    const double nn = static_cast<double>(kNC);
                    pp[0] = nn;
                    if constexpr (OUT == OUT_FLOAT_MOMENTS) {
                        pp[1] = t1 / nn;
                        pp[2] = t2 - t1 * (t1 / nn);
                    } else {
                        pp[1] = t1;
                        pp[2] = t2;
                    }
                }
                team_sync();  // red reusable
                d1 = d2 = 0.0;
                f1 = f2 = 0.f;
            }
        };

        // The part of an item after its input step: three GEMM stages, their
        // epilogues, the output.  The item is read before this warp's stage-3
        // publish in a chain (the leader writes the next item's slot only
        // after the stage-3 MMAs, which wait for every warp's publish).
        auto item_body = [&](int64_t item_static) {
            publish();
            wait_mma();
            epi1(h);
            epi1(h + 2);
            publish();
            wait_mma();
            epi2(h);
            epi2(h + 2);
            const int64_t item = CHAIN ? static_cast<int64_t>(slots[t]) : item_static;
            publish();
            const SegInv &s = a.s[seg_index(a, item)];
            const int64_t local = item - s.item0;
            const int64_t pol = local >= s.n ? 1 : 0, loc = local - pol * s.n;
            wait_mma();
#pragma unroll 1
            for (int j = h; j < 8; j += 2) epi3(j, s, pol, loc);
            if constexpr (OUT == OUT_TS_HALF) {  // the time series (64 KB, natural order) to global
                fence_async_smem();
                team_sync();
                if (et == 0) {
                    if (CHAIN && slots[18 + t] >= 0) {
                        // chain: the last item's series, stored an item ago, is
                        // complete in global memory: stage B may read its
                        // batch.  Signalled here, where no store or load of
                        // this thread is in flight.
                        bulk_wait_all();
                        fence_proxy_global();
                        bump(sc.done + slots[18 + t] / kBatchSnaps);
                    }
                    bulk_s2g(static_cast<__half *>(s.out) + pol * s.out_pol_stride + loc * static_cast<int64_t>(kNA), X,
                             kNA * 2);
                    if (CHAIN) slots[18 + t] = item;
                }
            }
            if constexpr (kQuant) {  // the payload (8192 bytes, natural order) to global
                fence_async_smem();
                team_sync();
                if (et == 0)
                    bulk_s2g(s.o.out + pol * s.o.out_pol_stride + (s.o.pkt0 + loc) * s.o.pkt_stride + s.o.payload_off,
                             X, 8192);
            }
            chunk_stats(s, pol, loc);
            fence_before();  // tensor-memory reads done before the next item's stage-1 MMAs (after its publish)
        };

        if constexpr (!CHAIN) {
            // Static order: team t takes items b + m G, m = t, t + 2, ...; the
            // staging of the bins input is filled in item order (the team that
            // has read item m's bins starts the copy of item m + 1's).
            auto fetch_bins = [&](int64_t m) {
                if (item_of(m) >= a.n_items) return;
                fence_async_smem();
                bulk_g2s(stg_all, item_in(item_of(m)), kStgBins, &ctl.stg[m & 1]);
            };
            if constexpr (kBins) {
                if (t == 0 && et == 0) fetch_bins(0);
            } else {
                if (item_of(t) < a.n_items) prefetch(item_of(t));
                // team 1 starts once team 0 has written its first operand, so that
                // the teams' MMA waits fall in each other's CUDA-core steps
                if (t == 1 && !err_on() && !mbar_wait(&ctl.ready[0], 0, lim)) raise();
            }
            for (int64_t m = t; item_of(m) < a.n_items; m += 2) {
                const int64_t item = item_of(m);
                if constexpr (kBins) {
                    if (!err_on() && !mbar_wait(&ctl.stg[t], sph, lim)) raise();
                    sph ^= 1u;
                    if constexpr (kQuant) {  // the last item's payload has left X
                        if (et == 0) bulk_wait_read();
                        team_sync();
                    }
                    input_row(et);
                    input_row(et + 256);
                    team_sync();  // staging read: it takes the next item's bins
                    if (et == 0) fetch_bins(m + 1);
                    // this team's next bins to L2, so that their copy into the staging
                    // (once the other team has read item m + 1's) reads L2, not HBM
                    if (et < 5 && item_of(m + 2) < a.n_items) l2_prefetch_piece(item_in(item_of(m + 2)), kStgBins, et);
                } else {
                    if (OUT == OUT_TS_HALF && et == 0) bulk_wait_read();  // the last item's series has left X
                    land();
                    // the team's next snapshot into registers now, a whole item ahead of its use
                    if (item_of(m + 2) < a.n_items) prefetch(item_of(m + 2));
                    team_sync();
                    input_n3(e, std::true_type{});
                    input_n3(15 - e, std::false_type{});
                }
                item_body(item);
            }
            if ((OUT == OUT_TS_HALF || kQuant) && et == 0) bulk_wait_all();
        } else {
            // Chain: stage A's pair j % 2 holds the team's item j and item j + 1,
            // and its leader holds the ticket after those (pend), taken an item
            // ahead so the ticket's latency stays off the critical path; stage
            // C's item of the team's fill is read after the staging barrier.
            // After the last item the issuer gets the end mark.
            int64_t pend = -1;
            int fs = t;
            if constexpr (!kBins) {
                if (et == 0) {
                    slots[18 + t] = -1;
                    slots[2 + 4 * t] = ticket_a();
                    slots[2 + 4 * t + 1] = ticket_a();
                    pend = ticket_a();
                }
                team_sync();
                if (slots[2 + 4 * t] >= 0) prefetch(slots[2 + 4 * t]);
                if (t == 1 && !err_on() && !mbar_wait(&ctl.ready[0], 0, lim)) raise();
            }
            for (int j = 0;; ++j) {
                if constexpr (kBins) {
                    if (!err_on() && !mbar_wait(&ctl.stg[t], sph, lim)) raise();
                    sph ^= 1u;
                    const int64_t item = slots[10 + (fs & 3)];
                    if (item < 0) break;
                    if (et == 0) slots[t] = item;
                    if constexpr (kQuant) {  // the last item's payload has left X
                        if (et == 0) bulk_wait_read();
                        team_sync();
                    }
                    input_row(et);
                    input_row(et + 256);
                    team_sync();  // staging read (the issuer makes the next fill after the publish)
                    fs += 2;
                } else {
                    const int pa = 2 + 4 * t + 2 * (j & 1);
                    const int64_t item = slots[pa];
                    if (item < 0) break;
                    if (OUT == OUT_TS_HALF && et == 0) bulk_wait_read();  // the last item's series has left X
                    land();
                    // the team's next snapshot into registers now, a whole item ahead of its use
                    if (slots[pa + 1] >= 0) prefetch(slots[pa + 1]);
                    if (et == 0) {
                        slots[t] = item;
                        const int pb = 2 + 4 * t + 2 * ((j + 1) & 1);
                        slots[pb] = slots[pa + 1];
                        slots[pb + 1] = pend;
                        pend = pend >= 0 ? ticket_a() : -1;
                    }
                    team_sync();
                    input_n3(e, std::true_type{});
                    input_n3(15 - e, std::false_type{});
                }
                item_body(0);
            }
            // end mark for the team's issuer
            if (et == 0) slots[t] = -1;
            publish();
            if ((OUT == OUT_TS_HALF || kQuant) && et == 0) {
                bulk_wait_all();
                if (OUT == OUT_TS_HALF && slots[18 + t] >= 0) {
                    fence_proxy_global();
                    bump(sc.done + slots[18 + t] / kBatchSnaps);
                }
            }
        }
    }
    fence_before();
    __syncthreads();
    if (threadIdx.x == 0 && *reinterpret_cast<const volatile int *>(&ctl.err) != 0)
        *reinterpret_cast<volatile int *>(a.status) = 1;
}

template <int IN, int OUT>
__global__ void __launch_bounds__(kInvThreads, 1) k_tcf_inv(const __grid_constant__ ArgsInv a) {
    extern __shared__ __align__(1024) uint8_t smem_raw[];
    uint8_t *sm = smem_raw + ((1024u - (smem_u32(smem_raw) & 1023u)) & 1023u);
    const int warp = threadIdx.x >> 5;
    if (warp == 0) tmem_alloc_cols(&g_tmem_base);
    fence_before();
    __syncthreads();
    fence_after();
    const uint32_t tb = g_tmem_base;
    inv_phase<IN, OUT, 0, false>(a, Sched{nullptr, nullptr, nullptr}, sm, tb);
    if (warp == 0) tmem_free_cols(tb);
}

// ============================================================================
// k_tcf_fwd: stage B, R2C 36608 per chunk -> bins [skip, skip + 16384]
// ============================================================================
// Index maps (N = 18304 = 143 x 128): n = (128 nA + 143 nB) mod N with
// nA = (13 n11 + 11 n13) mod 143 and nB = 8 n16 + n8; the output bin k has
// k mod 143 = kA with kA mod 11 = k11, kA mod 13 = k13, and k mod 128 =
// k16 + 16 k8, i.e. k = (2432 kA + 15873 kB) mod N.  Rows are labelled by
// nA' = 13 n11 + n13 (a relabelling of nA).
//   B1  DFT-16 over n16: rows 8 nA' + n8        (1144 in 9 tiles), K n16 (64-byte swizzle)
//       twiddle W_128^(n8 k16)
//   B2  DFT-8 over n8:   rows 144 k16 + nA'     (2304 in 18 tiles, nA' = 143 unused), K n8 (32-byte swizzle)
//   B3  DFT-11 over n11: rows n13 + 13 kB       (1664 in 13 tiles), K n11 (3 core matrices)
//   B4  DFT-13 over n13: rows 128 k11 + kB      (1408 in 11 tiles), K n13 (64-byte swizzle)
//   Z[k] in natural order -> R2C pairing -> bins [skip, skip + 16384] (FP16) to global.
struct SegFwd {
    const __half *in;        // time series x 2^-2, [pol][chunks][36608]
    uint32_t *out;           // bins (half2) [pol][chunks][kTcfBinsLen]
    int64_t in_pol_stride;   // halves
    int64_t out_pol_stride;  // bins
    int64_t n, item0;        // chunks per pol
    int skip;
    int64_t dep0;            // chain: stage-A batch counter of the segment's first batch (pol 0)
};
struct ArgsFwd {
    int64_t n_items;
    int n;
    SegFwd s[kMaxSegs];
    const uint8_t *g;        // forward DFT-16, DFT-8, DFT-11, DFT-13 matrices, pre-tiled
    const float2 *tab;       // the kFwdTabLen twiddle values
    int *status;
    uint64_t wait_ns;        // bound of every mbarrier wait
};

// One stage-B loop over its items (a whole k_tcf_fwd launch, or a phase of
// k_tcf_chain): warps 0-16 work, further warps of the block only join the
// CTA barriers.  Ends with a CTA barrier and every MMA retired.
template <bool CHAIN>
__device__ __forceinline__ void fwd_phase(const ArgsFwd &a, const Sched sc, uint8_t *sm, uint32_t tmem_base) {
    Ctl &ctl = g_ctl_fwd;
    volatile int64_t *slots = g_slots;
    uint8_t *X0 = sm, *X1 = sm + kFwdX0;
    float2 *tab = reinterpret_cast<float2 *>(sm + kFwdOffTab);
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;

    if (tid == 0) ctl_init(ctl, a.wait_ns);
    if (tid < kThreads) {
        const uint4 *src = reinterpret_cast<const uint4 *>(a.g);
        uint4 *dst = reinterpret_cast<uint4 *>(sm + kFwdOffG);
        for (int i = tid; i < static_cast<int>((kG16f + kG8f + kG11f + kG13f) / 16); i += kThreads)
            dst[i] = __ldg(src + i);
        for (int i = tid; i < kFwdTabLen; i += kThreads) tab[i] = __ldg(a.tab + i);
        // operands start finite (padding rows and K columns are read, against zero G entries)
        uint4 *z = reinterpret_cast<uint4 *>(sm);
        for (int i = tid; i < static_cast<int>((kFwdX0 + kFwdX1) / 16); i += kThreads) z[i] = make_uint4(0, 0, 0, 0);
    }
    fence_async_smem();
    fence_before();
    __syncthreads();
    fence_after();
    const uint32_t tb = tmem_base;
    auto item_pos = [&](int64_t item, int64_t &pol, int64_t &loc) -> int {
        const int si = seg_index(a, item);
        const int64_t local = item - a.s[si].item0;
        pol = local >= a.s[si].n ? 1 : 0;
        loc = local - pol * a.s[si].n;
        return si;
    };
    auto chunk_in = [&](int64_t z) -> const __half * {  // the item's 36608 FP16 samples
        int64_t pol, loc;
        const SegFwd &s = a.s[item_pos(z, pol, loc)];
        return s.in + pol * s.in_pol_stride + loc * static_cast<int64_t>(kNB);
    };

    if (warp == 0) {
        Issuer is{&ctl, tb};
        const uint32_t g16 = smem_u32(sm + kFwdOffG), g8 = g16 + kG16f, g11 = g8 + kG8f, g13 = g11 + kG11f;
        const uint32_t x0 = smem_u32(X0), x1 = smem_u32(X1);
        auto rest = [&]() {
            is.stage_all<1>(0, x0, 18, 4096, 32, 16, 256, kSwizzle32, g8, 256, 512, 16, 16);      // DFT-8
            is.stage_all<2>(1, x1, 13, 6144, 256, 128, 384, kNoSwizzle, g11, 512, 2048, 32, 32);  // DFT-11
            is.stage_all<2>(0, x0, 11, 8192, 32, 16, 512, kSwizzle64, g13, 512, 2048, 32, 32);    // DFT-13
        };
        if constexpr (CHAIN) {
            // The issuer also feeds the chain, in its idle time between MMA
            // stages (lane 0): the CTA's items as tickets (one taken ahead,
            // its chunk prefetched to L2), each item's wait for its stage-A
            // batch and the copy of its chunk into X0 once the last item's
            // DFT-13 MMAs have retired, and the completion signal of the last
            // item's bins once the epilogue has moved on.  Slot 14 + k % 2
            // tells the epilogue the k-th item (-1: end).
            auto ticket = [&]() -> int64_t {
                const int64_t z = static_cast<int64_t>(atomicAdd(sc.ticket, 1u));
                return z < a.n_items ? z : -1;
            };
            auto feed = [&](int64_t k, int64_t z) {
                slots[14 + (k & 1)] = z;
                if (z < 0) {
                    mbar_arrive(&ctl.stg);
                    return;
                }
                int64_t pol, loc;
                const SegFwd &s = a.s[item_pos(z, pol, loc)];
                const unsigned *d = sc.dep + s.dep0 + pol * (s.n / kChunks) + loc / kChunks;
                if (!err_set(ctl) && !wait_count(d, static_cast<unsigned>(kBatchSnaps), ctl.lim)) raise_err(ctl);
                fence_proxy_global();
                bulk_g2s(X0, chunk_in(z), kNB * 2, &ctl.stg);
            };
            auto prefetch_l2 = [&](int64_t z) {
                if (z >= 0)
                    for (int i = 0; i < 5; ++i) l2_prefetch_piece(chunk_in(z), kNB * 2, i);
            };
            int64_t cur = -1, pend = -1, prev = -1;
            if (lane == 0) {
                cur = ticket();
                feed(0, cur);
                pend = cur >= 0 ? ticket() : -1;
                prefetch_l2(pend);
            }
            cur = __shfl_sync(0xffffffffu, cur, 0);
            uint32_t b13ph = 0;
            for (int64_t k = 0;; ++k) {
                if (cur < 0) {  // the epilogue's end mark follows its last item
                    if (!err_set(ctl) && !mbar_wait(&ctl.ready[1], (is.rphase >> 1) & 1u, ctl.lim)) raise_err(ctl);
                    is.rphase ^= 2u;
                    if (lane == 0 && prev >= 0) bump(sc.done + prev);
                    __syncwarp();
                    break;
                }
                is.stage_all<2>(1, x1, 9, 8192, 32, 16, 512, kSwizzle64, g16, 512, 2048, 32, 32);  // DFT-16
                // the epilogue has finished the last item (its bins are written): signal them
                if (lane == 0 && prev >= 0) bump(sc.done + prev);
                rest();
                commit_elect(&ctl.b13);
                if (!err_set(ctl) && !mbar_wait(&ctl.b13, b13ph, ctl.lim)) raise_err(ctl);
                b13ph ^= 1u;
                int64_t nxt = -1;
                if (lane == 0) {  // X0 is free: the next item's chunk
                    nxt = pend;
                    feed(k + 1, nxt);
                    pend = nxt >= 0 ? ticket() : -1;
                    prefetch_l2(pend);
                }
                __syncwarp();
                prev = cur;
                cur = __shfl_sync(0xffffffffu, nxt, 0);
            }
        } else {
            for (int64_t item = blockIdx.x; item < a.n_items; item += gridDim.x) {
                is.stage_all<2>(1, x1, 9, 8192, 32, 16, 512, kSwizzle64, g16, 512, 2048, 32, 32);  // DFT-16
                rest();
            }
        }
        is.finish();
    } else if (warp <= kEpiWarps) {
        Epi ep{&ctl, lane, (warp - 1) >> 2, warp & 3, (warp - 1) * 32 + lane,
               tb + (static_cast<uint32_t>((warp & 3) * 32) << 16)};
        const int e = warp - 1, q = ep.q, et = ep.et;
        const uint32_t *raw = reinterpret_cast<const uint32_t *>(X0);
        uint32_t *Z = reinterpret_cast<uint32_t *>(X1);

        // input step: raw (natural order) -> DFT-16 operand.  A warp writes the
        // 512-byte row group of one nA' (rows 8 nA' + n8): lane = (n8, 16-byte
        // chunk c of n16 = 4c .. 4c + 3).  Its i-th gather takes n16 = 4c +
        // (i + c) % 4, so that the 32 lanes' addresses (15 n8 + 24 ((i + c) % 4)
        // mod 32) fall in 32 banks; two conditional rotations put the four
        // values back in n16 order for one 16-byte store.
        auto input = [&]() {
            const int n8 = lane >> 2, c = lane & 3;
#pragma unroll 1
            for (int nAp = e; nAp < 143; nAp += kEpiWarps) {
                const int n11 = nAp / 13, n13 = nAp - 13 * n11;
                int nA = 13 * n11 + 11 * n13;
                nA -= nA >= 143 ? 143 : 0;
                nA -= nA >= 143 ? 143 : 0;
                int base = 128 * nA + 143 * n8 + 4576 * c;
                base -= base >= kMB ? kMB : 0;
                base -= base >= kMB ? kMB : 0;
                uint32_t v[4];
#pragma unroll
                for (int i = 0; i < 4; ++i) {
                    int n = base + 1144 * ((i + c) & 3);
                    n -= n >= kMB ? kMB : 0;
                    v[i] = raw[n];
                }
                if (c & 1) {
                    const uint32_t t = v[3];
                    v[3] = v[2];
                    v[2] = v[1];
                    v[1] = v[0];
                    v[0] = t;
                }
                if (c & 2) {
                    uint32_t t = v[0];
                    v[0] = v[2];
                    v[2] = t;
                    t = v[1];
                    v[1] = v[3];
                    v[3] = t;
                }
                *reinterpret_cast<uint4 *>(X1 + 512 * nAp + 64 * n8 + ((c ^ (n8 >> 1)) << 4)) =
                    make_uint4(v[0], v[1], v[2], v[3]);
            }
        };
        // B1: DFT-16 out (k16), rows 8 nA' + n8 -> B2 operand row 144 k16 + nA', K n8:
        // a thread's 16 stores are one address plus 4608 k16.  Twiddle 2^-8
        // W_128^(n8 k16) from the table: per load 8 consecutive entries (64 bytes,
        // distinct banks), 4 lanes each.
        auto epi1 = [&](int j, uint32_t t) {
            const int r = 128 * j + 32 * q + lane, nAp = r >> 3, n8 = r & 7;
            uint32_t r0[16], r1[16];
            tmem_ld16(t, r0);
            tmem_ld16(t + 16, r1);
            tmem_wait<16>(r0, r1);
            if (nAp < 143) {
                uint8_t *d0 = X0 + sw32_off(nAp, n8);
#pragma unroll
                for (int k16 = 0; k16 < 16; ++k16) {
                    const float2 y = cmul(acc2(k16 < 8 ? r0 : r1, k16 & 7), tab[kTabW128 + 8 * k16 + n8]);
                    *reinterpret_cast<uint32_t *>(d0 + 4608 * k16) = pack_half2(y.x, y.y);
                }
            }
        };
        // The same for k16 = 4 g .. 4 g + 3 only (group g's quarter of a tile's columns).
        auto epi1q = [&](int j, uint32_t t) {
            const int r = 128 * j + 32 * q + lane, nAp = r >> 3, n8 = r & 7;
            uint32_t r0[8];
            tmem_ld8(t + 8 * ep.grp, r0);
            tmem_wait1<8>(r0);
            if (nAp < 143) {
                uint8_t *d0 = X0 + sw32_off(nAp, n8) + 4608 * 4 * ep.grp;
#pragma unroll
                for (int i = 0; i < 4; ++i) {
                    const int k16 = 4 * ep.grp + i;
                    const float2 y = cmul(acc2(r0, i), tab[kTabW128 + 8 * k16 + n8]);
                    *reinterpret_cast<uint32_t *>(d0 + 4608 * i) = pack_half2(y.x, y.y);
                }
            }
        };
        // B2: DFT-8 out (k8), rows 144 k16 + nA' -> B3 operand row n13 + 13 (k16 + 16 k8), K n11:
        // 208 rows (26 row groups of 384 bytes) per k8
        auto epi2 = [&](int j, uint32_t t) {
            const int r = 128 * j + 32 * q + lane;
            const int k16 = r / 144, nAp = r - 144 * k16, n11 = nAp / 13, n13 = nAp - 13 * n11;
            uint32_t r0[16];
            tmem_ld16(t, r0);
            tmem_wait1<16>(r0);
            uint8_t *d0 = X1 + k24_off(n13 + 13 * k16, n11);
            if (nAp < 143) {
#pragma unroll
                for (int k8 = 0; k8 < 8; ++k8) {
                    const float2 v = acc2(r0, k8);
                    *reinterpret_cast<uint32_t *>(d0 + 9984 * k8) = pack_half2(v.x, v.y);
                }
            }
        };
        // B3: DFT-11 out (k11), rows n13 + 13 kB -> B4 operand row 128 k11 + kB, K n13
        auto epi3 = [&](int j, uint32_t t) {
            const int r = 128 * j + 32 * q + lane, kB = r / 13, n13 = r - 13 * kB;
            uint32_t r0[16], r1[16];
            tmem_ld16(t, r0);       // k11 = 0..7
            tmem_ld16(t + 16, r1);  // k11 = 8..10 (+ zero columns)
            tmem_wait<16>(r0, r1);
            uint8_t *d0 = X0 + sw64_off(kB, n13);
#pragma unroll
            for (int k11 = 0; k11 < 11; ++k11) {
                const float2 v = acc2(k11 < 8 ? r0 : r1, k11 & 7);
                *reinterpret_cast<uint32_t *>(d0 + 8192 * k11) = pack_half2(v.x, v.y);
            }
        };
        // B4: DFT-13 out (k13), rows 128 k11 + kB -> Z[k], k = (2432 kA + 15873 kB) mod N,
        // kA = (78 k11 + 66 k13) mod 143: k advances by 14080 per k13.
        auto epi4 = [&](int j, uint32_t t) {
            const int kB = 32 * q + lane;
            const int kA0 = (78 * j) % 143;
            int k = (2432 * kA0 + 15873 * kB) % kMB;
            uint32_t r0[16], r1[16];
            tmem_ld16(t, r0);
            tmem_ld16(t + 16, r1);
            tmem_wait<16>(r0, r1);
#pragma unroll
            for (int k13 = 0; k13 < 13; ++k13) {
                const float2 v = acc2(k13 < 8 ? r0 : r1, k13 & 7);
                Z[k] = pack_half2(v.x, v.y);
                k += 14080;
                k -= k >= kMB ? kMB : 0;
            }
        };
        // R2C pairing: bins q = skip + jj, jj = 0..16384, from Z[q], Z[N - q];
        // half of each bin (stage C's C2R pairing factor), FP16 to global.  A
        // thread takes two consecutive bins per step (one 8-byte store); the
        // second twiddle is the first times W_36608.
        auto pair1 = [&](int qq) -> float2 {  // bin qq in {0, N}: real
            const float2 z0 = h2f(Z[0]);
            return make_float2(0.5f * (qq == 0 ? z0.x + z0.y : z0.x - z0.y), 0.f);
        };
        // y = (za + conj zb) / 4 - i w (za - conj zb) / 4 with w4 = w / 4
        auto pairw = [&](float2 za, float2 zb, float2 w4) -> float2 {
            const float s1 = za.x + zb.x, s2 = za.y - zb.y, d1 = za.x - zb.x, d2 = za.y + zb.y;
            return make_float2(fmaf(w4.x, d2, fmaf(w4.y, d1, 0.25f * s1)), fmaf(-w4.x, d1, fmaf(w4.y, d2, 0.25f * s2)));
        };
        auto pairing = [&](const SegFwd &s, int64_t pol, int64_t loc) {
            uint32_t *yo = s.out + pol * s.out_pol_stride + loc * static_cast<int64_t>(kTcfBinsLen);
            const float2 w1 = tab[kTabQLo + 1];
            // W_36608^1024, the step of the twiddle recurrence between a thread's bins
            const float2 wstep = cmul(tab[kTabQHi + 8], make_float2(1.f, 0.f));
            int qq = s.skip + 2 * et;  // qq + 1 < N (skip <= 1920)
            float2 w = cmul(tab[kTabQHi + (qq >> 7)], tab[kTabQLo + (qq & 127)]);
            w = make_float2(0.25f * w.x, 0.25f * w.y);
#pragma unroll 2
            for (int jj = 2 * et; jj < kMA; jj += 2 * kEpiThreads, qq += 2 * kEpiThreads) {
                float2 za0, za1;
                if ((qq & 1) == 0) {  // skip = 8 trim_mhz is even: one 8-byte load
                    const uint2 za = *reinterpret_cast<const uint2 *>(Z + qq);
                    za0 = h2f(za.x);
                    za1 = h2f(za.y);
                } else {
                    za0 = h2f(Z[qq]);
                    za1 = h2f(Z[qq + 1]);
                }
                const float2 zb1 = h2f(Z[kMB - 1 - qq]);
                const float2 y0 = qq == 0 ? pair1(0) : pairw(za0, h2f(Z[kMB - qq]), w);
                const float2 y1 = pairw(za1, zb1, cmul(w, w1));
                __stcs(reinterpret_cast<uint2 *>(yo + jj), make_uint2(pack_half2(y0.x, y0.y), pack_half2(y1.x, y1.y)));
                w = cmul(w, wstep);
            }
            if (et == 0) {  // bin 16384
                const int q1 = s.skip + kMA;
                float2 y;
                if (q1 == kMB) {
                    y = pair1(q1);
                } else {
                    const float2 w0 = cmul(tab[kTabQHi + (q1 >> 7)], tab[kTabQLo + (q1 & 127)]);
                    y = pairw(h2f(Z[q1]), h2f(Z[kMB - q1]), make_float2(0.25f * w0.x, 0.25f * w0.y));
                }
                __stcs(yo + kMA, pack_half2(y.x, y.y));
            }
        };

        // An item from its landed chunk to Z complete (after_input() runs
        // between the input step and its publish), and then its R2C pairing.
        auto front = [&](auto after_input) {
            input();
            after_input();
            ep.publish_all(1);
            // B1: tiles 0-7 two per group, the ninth split by columns
            for (int j = ep.grp; j < 8; j += 4) {
                ep.wait_full(j);
                epi1(j, ep.tq + 32 * j);
            }
            ep.wait_full(8);
            epi1q(8, ep.tq + 32 * 8);
            ep.fbits ^= (1u << 9) - 1u;
            ep.publish_all(0);
            ep.stage_group(18, 16, 1, [&](int j, uint32_t t) { epi2(j, t); });
            ep.publish_all(1);
            ep.stage_group(13, 32, 3, [&](int j, uint32_t t) { epi3(j, t); });
            ep.publish_all(0);
            ep.stage_group(11, 32, 2, [&](int j, uint32_t t) { epi4(j, t); });
            fence_before();
            named_sync_epi();  // Z complete; every DFT-13 MMA retired: X0 takes the next chunk
        };
        auto back = [&](int64_t item) {
            int64_t pol, loc;
            const SegFwd &s = a.s[item_pos(item, pol, loc)];
            pairing(s, pol, loc);
            named_sync_epi();  // Z read: X1 takes the next input step; the bins are written
        };

        if constexpr (!CHAIN) {
            // static order: CTA b takes items b, b + G, ...
            auto fetch_static = [&](int64_t item) {  // the item's 36608 FP16 samples -> X0 (73,216 bytes)
                if (item >= a.n_items || et != 0) return;
                int64_t pol, loc;
                const SegFwd &s = a.s[item_pos(item, pol, loc)];
                fence_async_smem();
                bulk_g2s(X0, s.in + pol * s.in_pol_stride + loc * static_cast<int64_t>(kNB), kNB * 2, &ctl.stg);
            };
            if (blockIdx.x < a.n_items) fetch_static(blockIdx.x);
            for (int64_t item = blockIdx.x; item < a.n_items; item += gridDim.x) {
                ep.wait_staging();
                // the CTA's next chunk to L2 (five pieces), so that its copy into
                // X0 after this chunk's DFT-13 reads L2, not HBM
                if (et < 5 && item + gridDim.x < a.n_items) l2_prefetch_piece(chunk_in(item + gridDim.x), kNB * 2, et);
                front([] {});
                fetch_static(item + gridDim.x);
                back(item);
            }
        } else {
            for (int64_t k = 0;; ++k) {
                ep.wait_staging();
                const int64_t item = slots[14 + (k & 1)];
                if (item < 0) break;
                front([] {});
                back(item);
            }
            // end mark for the issuer
            ep.publish_all(1);
        }
    }
    fence_before();
    __syncthreads();
    if (threadIdx.x == 0 && err_set(ctl)) *reinterpret_cast<volatile int *>(a.status) = 1;
}

__global__ void __launch_bounds__(kThreads, 1) k_tcf_fwd(const __grid_constant__ ArgsFwd a) {
    extern __shared__ __align__(1024) uint8_t smem_raw[];
    uint8_t *sm = smem_raw + ((1024u - (smem_u32(smem_raw) & 1023u)) & 1023u);
    const int warp = threadIdx.x >> 5;
    if (warp == 0) tmem_alloc_cols(&g_tmem_base);
    fence_before();
    __syncthreads();
    fence_after();
    const uint32_t tb = g_tmem_base;
    fwd_phase<false>(a, Sched{nullptr, nullptr, nullptr}, sm, tb);
    if (warp == 0) tmem_free_cols(tb);
}

// Stages A, B and C of one wave in one persistent launch: every CTA runs the
// stage-A loop, then stage B's, then stage C's, each on tickets of its stage
// (q[0], q[1], q[2]); a stage-B item waits until its stage-A batch is
// complete (q[3 + batch] = 143 snapshots), a stage-C item until its stage-B
// item is (q[3 + n_batches + item] = 1).  q is zeroed before the launch.
struct ChainArgs {
    ArgsInv A;
    ArgsFwd B;
    ArgsInv C;
    unsigned *q;
    int64_t n_batches;
};

template <int OUTC>
__global__ void __launch_bounds__(kInvThreads, 1) k_tcf_chain(const __grid_constant__ ChainArgs c) {
    extern __shared__ __align__(1024) uint8_t smem_raw[];
    uint8_t *sm = smem_raw + ((1024u - (smem_u32(smem_raw) & 1023u)) & 1023u);
    const int warp = threadIdx.x >> 5;
    if (warp == 0) tmem_alloc_cols(&g_tmem_base);
    fence_before();
    __syncthreads();
    fence_after();
    const uint32_t tb = g_tmem_base;
    unsigned *dep_a = c.q + 3, *done_b = c.q + 3 + c.n_batches;
    inv_phase<IN_PACKED, OUT_TS_HALF, 0, true>(c.A, Sched{c.q, nullptr, dep_a}, sm, tb);
    fwd_phase<true>(c.B, Sched{c.q + 1, dep_a, done_b}, sm, tb);
    inv_phase<IN_BINS, OUTC, 1, true>(c.C, Sched{c.q + 2, done_b, nullptr}, sm, tb);
    if (warp == 0) tmem_free_cols(tb);
}

// Float time series -> FP16 x 2^-2 (sdbe_resample_chunks in this form).
__global__ void k_tcf_to_half(const float *__restrict__ in, uint32_t *__restrict__ out, int64_t n_pairs) {
    for (int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; i < n_pairs;
         i += static_cast<int64_t>(gridDim.x) * blockDim.x) {
        const float2 v = reinterpret_cast<const float2 *>(in)[i];
        out[i] = pack_half2(kScaleA * v.x, kScaleA * v.y);
    }
}

// ---- host side ------------------------------------------------------------

// Real form of the complex DFT matrix of size r (sign -1 forward, +1 inverse),
// split into FP16 hi and lo halves: N = np rows (hi at rows [0, 2r), lo at
// [lo_row, lo_row + 2r), zero elsewhere), K = kp columns (2r used), K-major in
// core-matrix order (8 rows x 16 bytes; 128 bytes between core matrices along
// K, (K / 8) * 128 between row groups).  Row 2 kk + t of a half is output
// component t (re, im) of bin kk; column 2 nn + u is input component u of
// element nn.
std::vector<__half> dft_matrix_hilo(int r, int sign, int kp, int lo_row, int np) {
    std::vector<__half> out(static_cast<size_t>(np) * kp, __float2half_rn(0.f));
    for (int kk = 0; kk < r; ++kk)
        for (int nn = 0; nn < r; ++nn) {
            const long long e = static_cast<long long>(kk) * nn % r;
            const double ang = sign * 2.0 * 3.14159265358979323846 * static_cast<double>(e) / r;
            const double c = std::cos(ang), s = std::sin(ang);
            const double vals[2][2] = {{c, -s}, {s, c}};  // [t][u]
            for (int t = 0; t < 2; ++t)
                for (int u = 0; u < 2; ++u) {
                    const double v = vals[t][u];
                    const __half hv = __float2half_rn(static_cast<float>(v));
                    const __half lv = __float2half_rn(static_cast<float>(v - static_cast<double>(__half2float(hv))));
                    for (int part = 0; part < 2; ++part) {
                        const int n = (part ? lo_row : 0) + 2 * kk + t, k = 2 * nn + u;
                        const size_t off =
                            static_cast<size_t>((n >> 3) * (kp / 8) * 64 + (k >> 3) * 64 + (n & 7) * 8 + (k & 7));
                        out[off] = part ? lv : hv;
                    }
                }
        }
    return out;
}

float2 cis(double num, double den, int sign = +1) {
    const double ang = sign * 2.0 * 3.14159265358979323846 * num / den;
    return make_float2(static_cast<float>(std::cos(ang)), static_cast<float>(std::sin(ang)));
}

template <class T>
void append(std::vector<uint8_t> &blob, const std::vector<T> &v) {
    const size_t o = blob.size();
    blob.resize(o + v.size() * sizeof(T));
    std::memcpy(blob.data() + o, v.data(), v.size() * sizeof(T));
}

constexpr size_t kInvGBytes = kG32Bytes + kG16Bytes, kFwdGBytes = kG16f + kG8f + kG11f + kG13f;
// blob: inverse matrices, inverse tables, forward matrices, forward tables
constexpr size_t kBlobInvTab = kInvGBytes, kBlobFwdG = kBlobInvTab + kInvTabLen * 8,
                 kBlobFwdTab = kBlobFwdG + kFwdGBytes, kBlobBytes = kBlobFwdTab + kFwdTabLen * 8;
static_assert(kBlobFwdG % 16 == 0 && kBlobFwdTab % 16 == 0, "16-byte aligned blob parts");

std::vector<uint8_t> build_blob() {
    std::vector<uint8_t> blob;
    append(blob, dft_matrix_hilo(32, +1, 64, 64, 128));
    append(blob, dft_matrix_hilo(16, +1, 32, 32, 64));
    std::vector<float2> ti(kInvTabLen, make_float2(0.f, 0.f));
    for (int i = 0; i <= 16; ++i) ti[kTabA1 + i] = cis(i, 64);
    for (int i = 0; i < 512; ++i) ti[kTabA2 + i] = cis(i, 32768);
    for (int i = 0; i < 512; ++i) ti[kTabB + i + (i >> 4)] = cis(i, 16384);
    for (int i = 0; i < 16; ++i) ti[kTabC + i] = cis(i, 512);
    append(blob, ti);
    append(blob, dft_matrix_hilo(16, -1, 32, 32, 64));
    append(blob, dft_matrix_hilo(8, -1, 16, 16, 32));
    append(blob, dft_matrix_hilo(11, -1, 32, 32, 64));
    append(blob, dft_matrix_hilo(13, -1, 32, 32, 64));
    std::vector<float2> tf(kFwdTabLen, make_float2(0.f, 0.f));
    for (int k16 = 0; k16 < 16; ++k16)
        for (int n8 = 0; n8 < 8; ++n8) {
            const float2 w = cis((n8 * k16) % 128, 128, -1);
            tf[kTabW128 + 8 * k16 + n8] = make_float2(kScaleB * w.x, kScaleB * w.y);
        }
    for (int i = 0; i < 144; ++i) tf[kTabQHi + i] = cis(128.0 * i, 36608, -1);
    for (int i = 0; i < 128; ++i) tf[kTabQLo + i] = cis(i, 36608, -1);
    append(blob, tf);
    return blob;
}

cudaError_t grid_for(int64_t n_items, unsigned *grid) {
    int dev = 0, sms = 1;
    cudaError_t e = cudaGetDevice(&dev);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    *grid = static_cast<unsigned>(n_items < sms ? n_items : sms);
    return e;
}

// Inverse transforms: two items per CTA at a time (one per team).
cudaError_t grid_for_teams(int64_t n_items, unsigned *grid) {
    cudaError_t e = grid_for((n_items + 1) / 2, grid);
    return e;
}

template <int IN, int OUT>
cudaError_t launch_inv(const ArgsInv &args, cudaStream_t st) {
    if (args.n_items <= 0) return cudaSuccess;
    unsigned grid = 0;
    cudaError_t e = grid_for_teams(args.n_items, &grid);
    constexpr uint32_t smem = inv_smem(IN == IN_BINS);
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(k_tcf_inv<IN, OUT>, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem));
    if (e != cudaSuccess) return e;
    k_tcf_inv<IN, OUT><<<grid, kInvThreads, smem, st>>>(args);
    return cudaGetLastError();
}

template <int OUTC>
cudaError_t launch_chain(const ChainArgs &args, cudaStream_t st) {
    if (args.A.n_items <= 0) return cudaSuccess;
    unsigned grid = 0;
    cudaError_t e = grid_for(args.B.n_items, &grid);  // every CTA finds stage-B and stage-C work
    constexpr uint32_t smem = inv_smem(true) > kFwdSmem ? inv_smem(true) : kFwdSmem;
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(k_tcf_chain<OUTC>, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem));
    if (e != cudaSuccess) return e;
    k_tcf_chain<OUTC><<<grid, kInvThreads, smem, st>>>(args);
    return cudaGetLastError();
}

cudaError_t launch_fwd(const ArgsFwd &args, cudaStream_t st) {
    if (args.n_items <= 0) return cudaSuccess;
    unsigned grid = 0;
    cudaError_t e = grid_for(args.n_items, &grid);
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(k_tcf_fwd, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(kFwdSmem));
    if (e != cudaSuccess) return e;
    k_tcf_fwd<<<grid, kThreads, kFwdSmem, st>>>(args);
    return cudaGetLastError();
}

const uint8_t *blob_of(const sdbe_resampler *h) { return static_cast<const uint8_t *>(h->tcf_tabs); }

constexpr uint64_t kWaitNs = 1000000000ull;  // 1 s: far above any legitimate wait
constexpr bool kFusedByDefault = true;        // stage_launches 0: one launch per wave

}  // namespace

// Tables of the fast tensor-core kernels and the time-out flag, on first use.
int tcf_prepare(sdbe_resampler *h, cudaStream_t st) {
    if (h->tcf_tabs) return SDBE_OK;
    if (!h->tc_status_host) {
        if (cudaHostAlloc(&h->tc_status_host, sizeof(int), cudaHostAllocMapped) != cudaSuccess) {
            cudaGetLastError();
            return fail(h, SDBE_ERR_NOMEM, "cannot allocate the tensor-core status flag");
        }
        *h->tc_status_host = 0;
        SDBE_CK(h, cudaHostGetDevicePointer(reinterpret_cast<void **>(&h->tc_status), h->tc_status_host, 0));
    }
    const std::vector<uint8_t> blob = build_blob();
    if (blob.size() != kBlobBytes) return fail(h, SDBE_ERR_STATE, "tensor-core table layout mismatch");
    if (cudaMalloc(&h->tcf_tabs, blob.size()) != cudaSuccess) {
        cudaGetLastError();
        return fail(h, SDBE_ERR_NOMEM, "cannot allocate the tensor-core tables");
    }
    SDBE_CK(h, cudaMemcpyAsync(h->tcf_tabs, blob.data(), blob.size(), cudaMemcpyHostToDevice, st));
    SDBE_CK(h, cudaStreamSynchronize(st));  // blob is freed on return
    return SDBE_OK;
}

// Stage A in the fast tensor-core form over several stream pairs in one
// launch: per segment, snapshots [snap0, snap0 + n_snaps) of n_pols pols of
// the packed spectra -> time series out + pol * out_pol_stride (elements),
// [n_snaps][32768] per pol, FP16 x 2^-2 (half_out) or FP32.
namespace {
void build_a(sdbe_resampler *h, const TcfASeg *segs, int n_segs, int n_pols, ArgsInv &A) {
    for (int i = 0; i < n_segs; ++i) {
        const TcfASeg &g = segs[i];
        SegInv s{};
        s.in = g.spec;
        s.out = g.out;
        s.in_pol_stride = g.spec_pol_stride;
        s.first = g.snap0;
        s.n = g.n_snaps;
        s.out_pol_stride = g.out_pol_stride;
        s.item0 = A.n_items;
        A.s[A.n++] = s;
        A.n_items += n_pols * g.n_snaps;
    }
    A.g = blob_of(h);
    A.tab = reinterpret_cast<const float2 *>(blob_of(h) + kBlobInvTab);
    A.status = h->tc_status;
    A.wait_ns = kWaitNs;
}
}  // namespace

int tcf_stage_a(sdbe_resampler *h, const TcfASeg *segs, int n_segs, int n_pols, bool half_out, cudaStream_t st) {
    if (n_segs < 1 || n_segs > kMaxSegs) return fail(h, SDBE_ERR_ARG, "bad segment count");
    if (int rc = tcf_prepare(h, st)) return rc;
    ArgsInv A{};
    build_a(h, segs, n_segs, n_pols, A);
    if (h->tc_test_timeout_ns > 0) {  // test hook: one withheld signal, short waits
        A.wait_ns = static_cast<uint64_t>(h->tc_test_timeout_ns);
        A.withhold = 1;
        h->tc_test_timeout_ns = 0;
    }
    SDBE_CK(h, (half_out ? launch_inv<IN_PACKED, OUT_TS_HALF>(A, st) : launch_inv<IN_PACKED, OUT_TS_FLOAT>(A, st)));
    return SDBE_OK;
}

// Stages B and C in the fast tensor-core form over several stream pairs: per
// segment n_chunks chunks of n_pols pols of FP16 time series (x 2^-2) -> R2C
// bins (scratch) -> the output `mode` asks for: 0 2-bit payload, 1 floats +
// per-chunk (n, mean, M2), 3 2-bit payload + per-chunk (n, sum, sum of
// squares), 5 floats.
namespace {
void build_bc(sdbe_resampler *h, const TcfBCSeg *segs, int n_segs, int n_pols, ArgsFwd &B, ArgsInv &C) {
    for (int i = 0; i < n_segs; ++i) {
        const TcfBCSeg &g = segs[i];
        B.s[B.n++] = SegFwd{static_cast<const __half *>(g.ts), g.bins, g.ts_pol_stride, g.bins_pol_stride, g.n_chunks,
                            B.n_items, g.skip};
        B.n_items += n_pols * g.n_chunks;
        SegInv s{};
        s.in = g.bins;
        s.in_pol_stride = g.bins_pol_stride;
        s.n = g.n_chunks;
        s.item0 = C.n_items;
        s.o = g.o;
        C.s[C.n++] = s;
        C.n_items += n_pols * g.n_chunks;
    }
    B.g = blob_of(h) + kBlobFwdG;
    B.tab = reinterpret_cast<const float2 *>(blob_of(h) + kBlobFwdTab);
    B.status = h->tc_status;
    B.wait_ns = kWaitNs;
    C.g = blob_of(h);
    C.tab = reinterpret_cast<const float2 *>(blob_of(h) + kBlobInvTab);
    C.status = h->tc_status;
    C.wait_ns = kWaitNs;
}
}  // namespace

int tcf_stage_bc(sdbe_resampler *h, const TcfBCSeg *segs, int n_segs, int n_pols, int mode, cudaStream_t st) {
    if (n_segs < 1 || n_segs > kMaxSegs) return fail(h, SDBE_ERR_ARG, "bad segment count");
    if (int rc = tcf_prepare(h, st)) return rc;
    ArgsFwd B{};
    ArgsInv C{};
    build_bc(h, segs, n_segs, n_pols, B, C);
    SDBE_CK(h, launch_fwd(B, st));
    switch (mode) {
        case 0: SDBE_CK(h, (launch_inv<IN_BINS, OUT_QUANT>(C, st))); break;
        case 1: SDBE_CK(h, (launch_inv<IN_BINS, OUT_FLOAT_MOMENTS>(C, st))); break;
        case 3: SDBE_CK(h, (launch_inv<IN_BINS, OUT_QUANT_SUMS>(C, st))); break;
        default: SDBE_CK(h, (launch_inv<IN_BINS, OUT_FLOAT>(C, st))); break;
    }
    return SDBE_OK;
}

// Whether a wave's three stages run as one persistent launch (the handle's
// stage_launches; the time-out test hook needs the separate launches).
bool tcf_fused(const sdbe_resampler *h) {
    if (h->tc_test_timeout_ns > 0) return false;
    return h->cfg.stage_launches == SDBE_STAGES_FUSED ||
           (h->cfg.stage_launches == 0 && kFusedByDefault);
}

// One wave of the fast tensor-core chain over several handles (one stream
// pair each): stage A of every handle's batches in one launch (FP16 time
// series into the handle's stage-A scratch), then stages B and C in one launch
// each, writing the payloads; or all three stages in one persistent launch.  With `first` each item is its handle's first
// batch: stage C writes floats and FP64 moments, the thresholds are set from
// them, then the floats are packed, as the FP32 path does.
int tcf_wave_multi(const std::vector<TcWaveItem> &w, bool first, cudaStream_t st) {
    if (w.empty()) return SDBE_OK;
    if (w.size() > static_cast<size_t>(kMaxSegs)) return fail(w[0].h, SDBE_ERR_ARG, "too many handles");
    sdbe_resampler *h0 = w[0].h;
    std::vector<TcfASeg> sa;
    std::vector<TcfBCSeg> sb;
    int64_t units_a = 0, units_bc = 0;
    bool any_win = false;
    for (const auto &it : w) {
        sdbe_resampler *h = it.h;
        if (int rc = tcf_prepare(h, st)) return rc;
        if (*reinterpret_cast<volatile int *>(h->tc_status_host))  // written by an earlier call's kernels
            return fail(h, SDBE_ERR_CUDA, "a tensor-core transform timed out on its mbarrier wait");
        const int64_t per_pol = static_cast<int64_t>(h->wave) * kChunks;
        if (int rc = grow(h, reinterpret_cast<uint8_t **>(&h->tcf_bins), &h->tcf_bins_bytes,
                          2 * per_pol * kTcfBinsLen * 4, "the tensor-core bins"))
            return rc;
        const int64_t snaps = it.nb * kBatchSnaps, chunks = it.nb * kChunks;
        sa.push_back(TcfASeg{it.spec, it.spec_pol_stride, it.b0 * kBatchSnaps, snaps, h->ts, h->ts_pol_stride});
        TcfBCSeg b{};
        b.ts = h->ts;  // FP16 in the float scratch: same element stride, half the bytes
        b.ts_pol_stride = h->ts_pol_stride;
        b.bins = h->tcf_bins;
        b.bins_pol_stride = per_pol * kTcfBinsLen;
        b.n_chunks = chunks;
        b.skip = h->skip;
        const bool win = h->cfg.threshold_mode == SDBE_THRESH_WINDOW;
        if (first) {
            b.o.fout = h->fout;
            b.o.fout_pol_stride = static_cast<int64_t>(kChunks) * kNC;
            b.o.partials = h->partials;
        } else {
            const PayloadTarget &t = it.tgt;
            b.o.out = t.base;
            b.o.out_pol_stride = t.pol_stride;
            b.o.pkt_stride = t.pkt_stride;
            b.o.payload_off = t.payload_off;
            b.o.pkt0 = it.b0 * kChunks;
            b.o.thr = h->thr;
            b.o.partials = win ? h->wpart : nullptr;
            any_win = any_win || win;
        }
        sb.push_back(b);
        units_a += 2 * snaps;
        units_bc += 2 * chunks;
    }
    const int n = static_cast<int>(w.size());
    size_t slot = 0;
    if (!first && tcf_fused(h0)) {
        // stages A, B and C in one persistent launch (k_tcf_chain), on tickets
        ChainArgs c{};
        build_a(h0, sa.data(), n, 2, c.A);
        build_bc(h0, sb.data(), n, 2, c.B, c.C);
        for (int i = 0; i < c.B.n; ++i) c.B.s[i].dep0 = c.A.s[i].item0 / kBatchSnaps;
        c.n_batches = c.A.n_items / kBatchSnaps;
        const int64_t words = 3 + c.n_batches + c.B.n_items;
        if (int rc = grow(h0, &h0->tcf_chain, &h0->tcf_chain_bytes, words * 4, "the stage-chain counters")) return rc;
        c.q = reinterpret_cast<unsigned *>(h0->tcf_chain);
        SDBE_CK(h0, cudaMemsetAsync(c.q, 0, static_cast<size_t>(words) * 4, st));
        SDBE_CK(h0, timed_begin(h0, 2, units_bc, st, &slot));
        SDBE_CK(h0, (any_win ? launch_chain<OUT_QUANT_SUMS>(c, st) : launch_chain<OUT_QUANT>(c, st)));
        SDBE_CK(h0, timed_end(h0, slot, st));
        h0->launches -= 2;  // one launch instead of three (counted below)
    } else {
    if (!first) SDBE_CK(h0, timed_begin(h0, 0, units_a, st, &slot));
    if (int rc = tcf_stage_a(h0, sa.data(), n, 2, true, st)) return rc;
    if (!first) {
        SDBE_CK(h0, timed_end(h0, slot, st));
        SDBE_CK(h0, timed_begin(h0, 1, units_bc, st, &slot));
    }
    if (int rc = tcf_stage_bc(h0, sb.data(), n, 2, first ? 1 : (any_win ? 3 : 0), st)) return rc;
    }
    WinUpds U{};
    for (const auto &it : w) {
        sdbe_resampler *h = it.h;
        if (first) {
            SDBE_CK(h, launch_finalize_thresholds(h->partials, kChunks, h->cfg.pol1_uses_pol0_threshold, h->thr, st));
            const PayloadTarget &t = it.tgt;
            SDBE_CK(h, launch_quantize_chunks(h->fout, static_cast<int64_t>(kChunks) * kNC, kChunks, h->thr, t.base,
                                              t.pol_stride, t.pkt_stride, t.payload_off, it.b0 * kChunks, st));
            h->thresholds_set = true;
            h->stream_batch = 0;
            h->launches += 2;
        }
        // the window ring takes the wave's statistics after it was packed with the old thresholds
        window_step(h, first ? h->partials : h->wpart, it.nb, first, U);
    }
    if (U.n) {
        SDBE_CK(h0, launch_window_update(U, st));
        h0->launches += 1;
    }
    if (!first) SDBE_CK(h0, timed_end(h0, slot, st));
    h0->launches += 3;  // stage A, stage B, stage C
    return SDBE_OK;
}

cudaError_t tcf_to_half(const float *in, void *out, int64_t n_floats, cudaStream_t st) {
    k_tcf_to_half<<<1216, 256, 0, st>>>(in, static_cast<uint32_t *>(out), n_floats / 2);
    return cudaGetLastError();
}

}  // namespace sdbe

using namespace sdbe;

extern "C" int sdbe_test_tc_timeout(sdbe_resampler *h, int64_t limit_ns) {
    if (!h) return SDBE_ERR_ARG;
    if (limit_ns < 1000 || limit_ns > 1000000000) return fail(h, SDBE_ERR_ARG, "limit_ns must be in [1e3, 1e9]");
    if (h->cfg.precision != SDBE_PRECISION_TC16_FAST)
        return fail(h, SDBE_ERR_STATE, "the time-out test hook needs SDBE_PRECISION_TC16_FAST");
    h->tc_test_timeout_ns = limit_ns;
    return SDBE_OK;
}
