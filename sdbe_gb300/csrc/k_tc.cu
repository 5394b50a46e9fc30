// Precision form of the resampling stage on the 5th-generation tensor cores:
// every DFT block is a batched FP16 GEMM with FP32 accumulation in tensor
// memory (tcgen05.mma, operands in shared memory).  The DFT matrix is split
// into hi + lo FP16 halves; with SDBE_PRECISION_TC16 the data too (three
// products: hi*hi + hi*lo + lo*hi), with SDBE_PRECISION_TC16_FAST the data is
// rounded to FP16 (two products).
//
// A complex transform of length 128*N2 (16384 = 128*128 for the inverse
// transforms of stages A and C, 18304 = 128*143 for the forward transform of
// stage B) runs as the four-step factorisation, with n = N2*n1 + n2 and
// k = k1 + 128*k2 (NP = N2 rounded up to 16):
//   step 1  A[k1][n2] = sum_n1 F128[k1][n1] x[N2 n1 + n2]     GEMM 128 x NP, K = 128
//   step 2  B[k1][n2] = A[k1][n2] w^(n2 k1)                   twiddles, FP32
//   step 3  X[k1 + 128 k2] = sum_n2 B[k1][n2] F_N2[k2][n2]     GEMM 128 x NP, K = NP
// Complex products are real GEMMs accumulated into two TMEM accumulators
// (Dr = Fr Br - Fi Bi, Di = Fi Br + Fr Bi; the inverse flips the signs of
// the Fi terms through the instruction descriptor's negate-A bit).  Each
// transform's input is scaled by a power of two from its maximum and the
// step-1 output by a fixed power of two (exact) so that every FP16 half
// stays below 2^14.  The Hermitian pairings, the statistics and the 2-bit
// packing stay on the CUDA cores.
#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include <cmath>
#include <vector>

#include "fft_core.cuh"
#include "handle.cuh"

namespace sdbe {
namespace {

constexpr int kTcThreads = 256;
constexpr uint32_t kTmemCols = 512;
constexpr int kTile = 4096;  // one [128 rows][16 k] FP16 operand tile, core-matrix order

__device__ __forceinline__ uint32_t smem_u32(const void *p) { return static_cast<uint32_t>(__cvta_generic_to_shared(p)); }

// Shared-memory matrix descriptor, no swizzle, K-major: core matrices of 8
// rows x 16 bytes stored contiguously; LBO = byte step between core matrices
// along K, SBO = byte step along M/N.
__device__ __forceinline__ uint64_t smem_desc(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
    return static_cast<uint64_t>((saddr >> 4) & 0x3FFFu) | (static_cast<uint64_t>((lbo >> 4) & 0x3FFFu) << 16) |
           (static_cast<uint64_t>((sbo >> 4) & 0x3FFFu) << 32) | (1ull << 46);
}

// Instruction descriptor, kind::f16: F32 accumulator, F16 A and B, both K-major.
__device__ __forceinline__ uint32_t instr_desc(int m, int n, bool neg_a) {
    return (1u << 4) | (neg_a ? (1u << 13) : 0u) | (static_cast<uint32_t>(n >> 3) << 17) |
           (static_cast<uint32_t>(m >> 4) << 24);
}

__device__ __forceinline__ void mma_f16(uint32_t d_tmem, uint64_t a, uint64_t b, uint32_t idesc, bool acc) {
    asm volatile(
        "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
        " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(d_tmem),
        "l"(a), "l"(b), "r"(idesc), "r"(acc ? 1u : 0u));
}

// Eight columns at ta and eight at tb (this thread's lane), one wait for both;
// the wait names the registers so that no use moves above it.
__device__ __forceinline__ void tmem_ld8x2(uint32_t ta, uint32_t tb, float *va, float *vb) {
    uint32_t r[16];
    asm volatile("tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7])
                 : "r"(ta));
    asm volatile("tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
                 : "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]),
                   "=r"(r[15])
                 : "r"(tb));
    asm volatile("tcgen05.wait::ld.sync.aligned;"
                 : "+r"(r[0]), "+r"(r[1]), "+r"(r[2]), "+r"(r[3]), "+r"(r[4]), "+r"(r[5]), "+r"(r[6]), "+r"(r[7]),
                   "+r"(r[8]), "+r"(r[9]), "+r"(r[10]), "+r"(r[11]), "+r"(r[12]), "+r"(r[13]), "+r"(r[14]),
                   "+r"(r[15])::"memory");
#pragma unroll
    for (int i = 0; i < 8; ++i) {
        va[i] = __uint_as_float(r[i]);
        vb[i] = __uint_as_float(r[8 + i]);
    }
}

// Eight TMEM columns of this thread's lane into r, no wait (see tmem_wait_tied).
__device__ __forceinline__ void tmem_ld8_nw(uint32_t taddr, uint32_t *r) {
    asm volatile("tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7])
                 : "r"(taddr));
}

// Waits for this thread's TMEM loads; then ties each register of a[0..N) and
// b[0..N) to an (empty) asm after the wait, so that no use moves above it.
template <int N>
__device__ __forceinline__ void tmem_wait_tied(uint32_t *a, uint32_t *b) {
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int i = 0; i < N; i += 8) {
        asm volatile("" : "+r"(a[i]), "+r"(a[i + 1]), "+r"(a[i + 2]), "+r"(a[i + 3]), "+r"(a[i + 4]), "+r"(a[i + 5]),
                     "+r"(a[i + 6]), "+r"(a[i + 7]));
        asm volatile("" : "+r"(b[i]), "+r"(b[i + 1]), "+r"(b[i + 2]), "+r"(b[i + 3]), "+r"(b[i + 4]), "+r"(b[i + 5]),
                     "+r"(b[i + 6]), "+r"(b[i + 7]));
    }
}

// Bounded wait for the commit of phase `phase`; false on time-out.
__device__ __forceinline__ bool mbar_wait(uint64_t *mbar, uint32_t phase) {
    uint32_t done = 0;
    for (int it = 0; it < (1 << 22) && !done; ++it)
        asm volatile(
            "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
            : "=r"(done)
            : "r"(smem_u32(mbar)), "r"(phase & 1u));
    return done != 0;
}

// Byte offset of element (row, k) in a K-major operand with `kdim` columns.
__device__ __forceinline__ uint32_t op_off(int row, int k, int kdim) {
    return static_cast<uint32_t>((row >> 3) * (kdim / 8) * 128 + (k >> 3) * 128 + (row & 7) * 16 + (k & 7) * 2);
}

// 2^(14 - e) where maxabs < 2^e: the exact scale that brings |values| below 2^14.
__device__ __forceinline__ float pow2_scale(float maxabs) {
    if (!(maxabs > 0.f)) return 1.f;
    const int e = static_cast<int>((__float_as_uint(maxabs) >> 23) & 0xFFu) - 126;
    int s = 14 - e;
    s = s > 100 ? 100 : (s < -100 ? -100 : s);
    return __uint_as_float(static_cast<uint32_t>(127 + s) << 23);
}

__device__ __forceinline__ float block_max(float v, float *red) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = fmaxf(v, __shfl_xor_sync(0xffffffffu, v, o));
    __syncthreads();
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
    __syncthreads();
    float m = 0.f;
    for (int w = 0; w < kTcThreads / 32; ++w) m = fmaxf(m, red[w]);
    return m;
}

// One stream pair's transforms in a launch: 2 x per_pol items, pol-major,
// global items item0 .. item0 + 2 per_pol.
struct TcSeg {
    const float2 *in;
    int64_t in_stride, in_pol_stride;  // complex elements between items / between pols
    float2 *out;
    int64_t out_stride, out_pol_stride;
    int64_t per_pol, item0;
};

struct TcFftArgs {
    int64_t n_items;                   // items of all segments
    int n;                             // segments
    TcSeg s[kMaxSegs];
    const uint8_t *f1;                 // DFT-128 tiles [8 K-steps][4 comps][4 KB]
    const uint8_t *f2;                 // DFT-N2 tiles [K-steps][4 comps][NP rows x 16 k]
    const float2 *tw;                  // e^{-2 pi i e / (128 N2)}, e < 128 N2
    int *status;                       // set to 1 on a barrier time-out (host-mapped)
};

__device__ __forceinline__ const TcSeg &seg_of(const TcFftArgs &a, int64_t item) {
    int j = 0;
    while (j + 1 < a.n && item >= a.s[j + 1].item0) ++j;
    return a.s[j];
}

__device__ __forceinline__ void mbar_init(uint64_t *mbar) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(mbar)));
}

// Arrival of this thread + `bytes` expected from bulk copies, then the bulk
// copy global -> shared that delivers them.
__device__ __forceinline__ void bulk_load(void *dst, const void *src, uint32_t bytes, uint64_t *mbar) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(mbar)), "r"(bytes)
                 : "memory");
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(smem_u32(dst)),
        "l"(src), "r"(bytes), "r"(smem_u32(mbar))
        : "memory");
}

// A bulk copy global -> shared that reports its bytes to mbar (whose expected
// bytes were set by one arrive.expect_tx for several copies).
__device__ __forceinline__ void bulk_copy(void *dst, const void *src, uint32_t bytes, uint64_t *mbar) {
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(smem_u32(dst)),
        "l"(src), "r"(bytes), "r"(smem_u32(mbar))
        : "memory");
}

__device__ __forceinline__ void arrive_expect_tx(uint64_t *mbar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(mbar)), "r"(bytes) : "memory");
}

// The barrier completes when every tcgen05 operation this thread issued so far has.
__device__ __forceinline__ void mma_commit(uint64_t *mbar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(mbar))
                 : "memory");
}

__device__ __forceinline__ uint32_t pick4(uint32_t a, uint32_t b, uint32_t c, uint32_t d, int j) {
    const uint32_t lo = (j & 1) ? b : a, hi = (j & 1) ? d : c;
    return (j & 2) ? hi : lo;
}

// (a, b) -> FP16 pairs hi = rn(a, b), lo = rn(a - hi, b - hi) as 32-bit words.
__device__ __forceinline__ void split2(float a, float b, uint32_t &hi, uint32_t &lo) {
    const __half2 h = __floats2half2_rn(a, b);
    const float2 hf = __half22float2(h);
    const __half2 l = __floats2half2_rn(a - hf.x, b - hf.y);
    hi = *reinterpret_cast<const uint32_t *>(&h);
    lo = *reinterpret_cast<const uint32_t *>(&l);
}

// (a, b) -> the FP16 pair rn(a, b) as a 32-bit word.
__device__ __forceinline__ uint32_t hi2(float a, float b) {
    const __half2 h = __floats2half2_rn(a, b);
    return *reinterpret_cast<const uint32_t *>(&h);
}

template <int N2, int NS>
struct TcGeo {
    static constexpr int NP = (N2 + 15) / 16 * 16;  // N of both GEMMs, step-3 K
    static constexpr int KS3 = NP / 16;             // step-3 K-steps (step 1 has 8)
    static constexpr int SPI = 8 + KS3;             // pipeline stages (K-steps) per item
    static constexpr int RG = NP / 8;               // 8-row groups of the step-1 B operand
    static constexpr int NPAIR = NP * 64 / kTcThreads;  // input element pairs per thread
    static constexpr uint32_t COMP = NP * 128 * 2;  // bytes of one B-operand component
    // 16384 points with FP16 data (NS = 2): the data operand takes two
    // components (64 KB), so all eight DFT-128 stages stay resident (128 KB),
    // loaded once per CTA and read by both GEMMs
    static constexpr bool RES = N2 == 128 && NS == 2;
    static constexpr int NCOMP = NS == 3 ? 4 : 2;   // data components kept: re/im x hi/lo, or hi only
    static constexpr int NRING = RES ? 8 : 4;       // DFT-tile buffers
    static constexpr uint32_t STAGE1 = 4 * kTile;   // bytes of a step-1 stage: DFT-128 [128 rows][16 k] x 4
    static constexpr uint32_t STAGE3 = 4 * NP * 32; // bytes of a step-3 stage: DFT-N2 [NP rows][16 k] x 4
    static constexpr uint32_t STAGE = STAGE3 > STAGE1 ? STAGE3 : STAGE1;
    static constexpr size_t SMEM = NCOMP * static_cast<size_t>(COMP) + NRING * static_cast<size_t>(STAGE) +
                                   (N2 + 128) * sizeof(float2);
};

// One CTA per SM (its shared memory and all 512 TMEM columns), persistent
// over items.  Step 1 is D[k1][n2] = F128 (A) x B[n2][n1] (B operand); step 3
// is D[k1][k2] = B2[k1][n2] (A) x F_N2[k2][n2] (B operand), so both GEMMs are
// 128 x NP and step 3 leaves y[k1 + 128 k2] in TMEM lane k1, column k2, which
// a warp stores as 32 consecutive complex values.  Accumulators: Dr at column
// 0, Di at 256 (at 16384 points step 1 at 0 and 128, step 3 at 256 and 384,
// so that an output is stored while the next step-1 GEMM runs).  Thread 0
// issues the MMAs and the bulk copies of the DFT tiles through a ring of four
// buffers (the tiles of K-step g+3 load while the MMAs of K-step g run; all
// resident at 16384 points with FP16 data); warps 1-7 load the next item's
// input into registers while the current item's step-3 GEMM runs, warp 0
// (whose lane 0 issues) after it.
//
// Input element pairs: thread tid holds pairs i*256 + tid, i < NPAIR; pair p
// is row (q % RG)*8 + (p & 7) and K columns 2kp, 2kp+1 with q = p >> 5 and
// kp = (q / RG)*4 + ((p >> 3) & 3), so one warp's 32-bit stores cover whole
// 128-byte core-matrix rows: no bank conflicts.  Step 2 rotates the order of
// a row's four words by its row group for the same reason.
template <int N2, bool INV, int NS>
__global__ void __launch_bounds__(kTcThreads, 1) k_tc_fft(const __grid_constant__ TcFftArgs a) {
    using G = TcGeo<N2, NS>;
    constexpr bool RES = G::RES;
    // 16384 points: step 3 gets its own TMEM columns (Dr at 256, Di at 384;
    // step 1 at 0 and 128), so that one transform's output is stored while
    // the next one's step-1 GEMM runs.  18304 points need 288 columns a step.
    constexpr bool OVL = N2 == 128;
    constexpr uint32_t DI1 = OVL ? 128 : 256, D3 = OVL ? 256 : 0, DI3 = OVL ? 128 : 256;
    // physical slot of data component c (0 re hi, 1 re lo, 2 im hi, 3 im lo)
    auto cslot = [](int c) { return NS == 3 ? c : c >> 1; };
    constexpr int NP = G::NP, KS3 = G::KS3, SPI = G::SPI, RG = G::RG, NPAIR = G::NPAIR;
    constexpr int NRING = G::NRING;
    constexpr uint32_t COMP = G::COMP, STAGE = G::STAGE, STAGE1 = G::STAGE1, STAGE3 = G::STAGE3;
    extern __shared__ __align__(1024) uint8_t smem[];
    uint8_t *bop = smem;                                               // [NCOMP][COMP]
    uint8_t *aop = smem + G::NCOMP * COMP;                             // [NRING][STAGE]
    float2 *twh = reinterpret_cast<float2 *>(aop + NRING * STAGE);    // w^(128 i), i < N2
    float2 *twl = twh + N2;                                            // w^j, j < 128
    __shared__ __align__(8) uint64_t full[NRING], empty[NRING], done;
    __shared__ uint32_t tmem_base;
    __shared__ int s_err;
    __shared__ float red[kTcThreads / 32];
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int quarter = warp & 3, half = warp >> 2;

    if (tid == 0) {
        for (int b = 0; b < NRING; ++b) {
            mbar_init(&full[b]);
            mbar_init(&empty[b]);
        }
        mbar_init(&done);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        s_err = 0;
    }
    for (int i = tid; i < N2 + 128; i += kTcThreads) {  // step-2 twiddles w^e = twh[e >> 7] twl[e & 127]
        float2 w = __ldg(a.tw + (i < N2 ? 128 * i : i - N2));
        if (INV) w.y = -w.y;
        twh[i] = w;  // twl = twh + N2
    }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&tmem_base)),
                     "r"(kTmemCols));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t tb = tmem_base;
    const uint32_t lane_base = tb + (static_cast<uint32_t>(quarter * 32) << 16);

    // ---- issuer state (thread 0) ----------------------------------------------
    uint32_t g = 0;                      // global stage index (items x SPI)
    bool err = false;                    // a wait of thread 0 timed out: issue nothing more
    uint32_t pend = 0;                   // buffers with a bulk copy in flight
    uint32_t pend_g[NRING] = {};         // the stage each of those copies is for
    uint32_t done_n = 0;                 // completions of `done` waited for (all threads)

    auto issue_copy = [&](uint32_t gg) {
        const int64_t item = blockIdx.x + static_cast<int64_t>(gg / SPI) * gridDim.x;
        if (item >= a.n_items) return;
        const int kk = static_cast<int>(gg % SPI), b = gg % NRING;
        const uint8_t *src = kk < 8 ? a.f1 + kk * STAGE1 : a.f2 + (kk - 8) * STAGE3;
        bulk_load(aop + b * STAGE, src, kk < 8 ? STAGE1 : STAGE3, &full[b]);
        pend |= 1u << b;
        pend_g[b] = gg;
    };
    // One GEMM phase (thread 0), nst K-steps: step 1 (A = DFT-128 tiles from
    // the ring, B = the data in bop with K = 128) or step 3 (A = the data in
    // bop with K = NP, B = DFT-N2 tiles from the ring).
    auto gemm = [&](int nst, bool step3) {
        const uint32_t dr = tb + (step3 ? D3 : 0), di = dr + (step3 ? DI3 : DI1);
        const uint32_t idesc = instr_desc(128, NP, false), idesc_m = instr_desc(128, NP, true);
        for (int s = 0; s < nst; ++s, ++g) {
            const int b = RES ? s : g % NRING;  // resident tiles: K-step s in buffer s
            if (!RES && !err) {
                if (mbar_wait(&full[b], (g / NRING) & 1u))
                    pend &= ~(1u << b);
                else
                    err = true;
            }
            if (!err) {
                asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
                const uint8_t *ab = aop + b * STAGE;
#pragma unroll
                for (int q = 0; q < NS; ++q) {
                    // products (F hi, x hi), (F hi, x lo), (F lo, x hi); NS = 2 leaves out the second
                    const int sp = NS == 3 ? q : 2 * q;
                    const int fh = sp == 2 ? 1 : 0, xh = sp == 1 ? 1 : 0;
                    const bool first = s == 0 && q == 0;
                    if (!step3) {
                        const uint64_t fr = smem_desc(smem_u32(ab + (0 + fh) * kTile), 128, 256);
                        const uint64_t fi = smem_desc(smem_u32(ab + (2 + fh) * kTile), 128, 256);
                        const uint64_t xr = smem_desc(smem_u32(bop + cslot(0 + xh) * COMP) + s * 256, 128, 16 * 128);
                        const uint64_t xi = smem_desc(smem_u32(bop + cslot(2 + xh) * COMP) + s * 256, 128, 16 * 128);
                        // Dr += Fr Xr -/+ Fi Xi ; Di += +/-Fi Xr + Fr Xi
                        mma_f16(dr, fr, xr, idesc, !first);
                        mma_f16(dr, fi, xi, INV ? idesc : idesc_m, true);
                        mma_f16(di, fi, xr, INV ? idesc_m : idesc, !first);
                        mma_f16(di, fr, xi, idesc, true);
                    } else {
                        const uint64_t xr = smem_desc(smem_u32(bop + cslot(0 + xh) * COMP) + s * 256, 128, (NP / 8) * 128);
                        const uint64_t xi = smem_desc(smem_u32(bop + cslot(2 + xh) * COMP) + s * 256, 128, (NP / 8) * 128);
                        const uint64_t fr = smem_desc(smem_u32(ab + (0 + fh) * (NP * 32)), 128, 256);
                        const uint64_t fi = smem_desc(smem_u32(ab + (2 + fh) * (NP * 32)), 128, 256);
                        mma_f16(dr, xr, fr, idesc, !first);
                        mma_f16(dr, xi, fi, INV ? idesc : idesc_m, true);
                        mma_f16(di, xr, fi, INV ? idesc_m : idesc, !first);
                        mma_f16(di, xi, fr, idesc, true);
                    }
                }
            }
            if (!RES) mma_commit(&empty[b]);
            if (s == nst - 1) mma_commit(&done);
            if (!RES && !err) {
                // the buffer of K-step g-1 takes K-step g+3 once those MMAs are done
                if (g >= 1 && !mbar_wait(&empty[(g - 1) % NRING], ((g - 1) / NRING) & 1u)) err = true;
                if (!err) issue_copy(g + NRING - 1);
            }
        }
    };
    // All threads: the GEMM phase's accumulators are final.
    auto wait_done = [&]() {
        if (!mbar_wait(&done, done_n & 1u)) s_err = 1;
        ++done_n;
        __syncwarp();  // warp 0 reconverges before the warp-collective TMEM loads
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    };

    float2 xv[2 * NPAIR];
    auto load_input = [&](int64_t item) {
        const TcSeg &sg = seg_of(a, item);
        const int64_t local = item - sg.item0, pol = local / sg.per_pol, loc = local % sg.per_pol;
        const float2 *x = sg.in + pol * sg.in_pol_stride + loc * sg.in_stride;
#pragma unroll
        for (int i = 0; i < NPAIR; ++i) {
            const int q = i * 8 + warp;
            const int row = (q % RG) * 8 + (lane & 7);
            const int k = ((q / RG) * 4 + (lane >> 3)) * 2;
            xv[2 * i] = row < N2 ? __ldg(x + N2 * k + row) : make_float2(0.f, 0.f);
            xv[2 * i + 1] = row < N2 ? __ldg(x + N2 * (k + 1) + row) : make_float2(0.f, 0.f);
        }
    };

    if (tid == 0) {
        if constexpr (RES) {  // all eight K-step stages once; wait before the first GEMM
            arrive_expect_tx(&full[0], 8 * STAGE);
            for (int k = 0; k < 8; ++k) bulk_copy(aop + k * STAGE, a.f1 + k * STAGE, STAGE, &full[0]);
            pend = 1u;
            pend_g[0] = 0;
            if (blockIdx.x < a.n_items) {
                if (mbar_wait(&full[0], 0))
                    pend = 0;
                else
                    err = true;
            }
        } else {
            for (int i = 0; i < NRING - 1; ++i) issue_copy(i);
        }
    }
    // y[k1 + 128 k2] = step-3 result x inv, a warp's stores 32 consecutive values
    constexpr int HALF_OUT = NP / 2;
    auto store_out = [&](float2 *yo, float inv) {
        const int k1 = quarter * 32 + lane;
        for (int c0 = half * HALF_OUT; c0 < (half + 1) * HALF_OUT; c0 += 8) {
            float dr[8], di[8];
            tmem_ld8x2(lane_base + D3 + c0, lane_base + D3 + DI3 + c0, dr, di);
#pragma unroll
            for (int j = 0; j < 8; ++j)
                if (c0 + j < N2) __stcs(yo + k1 + 128 * (c0 + j), make_float2(dr[j] * inv, di[j] * inv));
        }
        asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    };
    float2 *y_prev = nullptr;  // OVL: the transform whose output is still in TMEM
    float inv_prev = 0.f;

    if (blockIdx.x < a.n_items) load_input(blockIdx.x);
    for (int64_t item = blockIdx.x; item < a.n_items; item += gridDim.x) {
        const TcSeg &sg = seg_of(a, item);
        const int64_t local = item - sg.item0;
        float2 *y = sg.out + (local / sg.per_pol) * sg.out_pol_stride + (local % sg.per_pol) * sg.out_stride;
        // ---- input: scaled below 2^14, split, B[n2][n1] -------------------------
        float m = 0.f;
#pragma unroll
        for (int i = 0; i < 2 * NPAIR; ++i) m = fmaxf(m, fmaxf(fabsf(xv[i].x), fabsf(xv[i].y)));
        const float s1 = pow2_scale(block_max(m, red));
#pragma unroll
        for (int i = 0; i < NPAIR; ++i) {
            const int q = i * 8 + warp;
            const int row = (q % RG) * 8 + (lane & 7);
            const int k = ((q / RG) * 4 + (lane >> 3)) * 2;
            const uint32_t off = op_off(row, k, 128);
            if constexpr (NS == 3) {
                uint32_t rh, rl, ih, il;
                split2(xv[2 * i].x * s1, xv[2 * i + 1].x * s1, rh, rl);
                split2(xv[2 * i].y * s1, xv[2 * i + 1].y * s1, ih, il);
                *reinterpret_cast<uint32_t *>(bop + off) = rh;
                *reinterpret_cast<uint32_t *>(bop + COMP + off) = rl;
                *reinterpret_cast<uint32_t *>(bop + 2 * COMP + off) = ih;
                *reinterpret_cast<uint32_t *>(bop + 3 * COMP + off) = il;
            } else {
                *reinterpret_cast<uint32_t *>(bop + off) = hi2(xv[2 * i].x * s1, xv[2 * i + 1].x * s1);
                *reinterpret_cast<uint32_t *>(bop + COMP + off) = hi2(xv[2 * i].y * s1, xv[2 * i + 1].y * s1);
            }
        }
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
        __syncthreads();
        // ---- step 1: D[k1][n2] -----------------------------------------------------
        if (tid == 0) gemm(8, false);
        if (OVL && y_prev) {  // the previous transform's output, beside this step-1 GEMM
            __syncwarp();     // warp 0 reconverges after its lane 0 issued
            store_out(y_prev, inv_prev);
        }
        wait_done();
        // ---- step 2: twiddles, scale, split into B[k1][n2] -----------------------
        // The scaled input is below 2^14 per component, so |D| < 128 sqrt(2) 2^14
        // < 2^21.5 and the twiddles keep magnitudes: the fixed scale 2^-8 keeps
        // every FP16 half below 2^14 without a pass for the maximum.  TMEM is
        // read GC chunks of 8 columns per wait.
        const int k1 = quarter * 32 + lane;
        constexpr int HALF = NP / 2, NCH = HALF / 8, GC = G::RES ? 4 : 1;  // one chunk where registers are short
        static_assert(NCH % GC == 0, "chunk groups");
        constexpr float s2 = 1.f / 256.f;
        const int rot = lane >> 3;  // = (k1 >> 3) & 3
#pragma unroll 1
        for (int cg = 0; cg < NCH; cg += GC) {
        uint32_t ur[8 * GC], ui[8 * GC];
#pragma unroll
        for (int q = 0; q < GC; ++q) {
            tmem_ld8_nw(lane_base + half * HALF + 8 * (cg + q), ur + 8 * q);
            tmem_ld8_nw(lane_base + DI1 + half * HALF + 8 * (cg + q), ui + 8 * q);
        }
        tmem_wait_tied<8 * GC>(ur, ui);
#pragma unroll
        for (int q = 0; q < GC; ++q) {
            const int c0 = half * HALF + 8 * (cg + q);
            float2 v[8];
#pragma unroll
            for (int j = 0; j < 8; ++j) {
                const int n2 = c0 + j;
                v[j] = make_float2(0.f, 0.f);
                if (n2 < N2) {
                    const int e = n2 * k1;  // < 128 N2
                    v[j] = cmul(make_float2(__uint_as_float(ur[8 * q + j]), __uint_as_float(ui[8 * q + j])),
                                cmul(twh[e >> 7], twl[e & 127]));
                }
            }
            uint32_t w[4][4];  // [component][word: columns 2j, 2j+1]
#pragma unroll
            for (int j = 0; j < 4; ++j) {
                split2(v[2 * j].x * s2, v[2 * j + 1].x * s2, w[0][j], w[1][j]);
                split2(v[2 * j].y * s2, v[2 * j + 1].y * s2, w[2][j], w[3][j]);
            }
#pragma unroll
            for (int t = 0; t < 4; ++t) {
                const int j = (t + rot) & 3;
                const uint32_t off = op_off(k1, c0 + 2 * j, NP);
#pragma unroll
                for (int c = 0; c < 4; ++c)
                    if (NS == 3 || (c & 1) == 0)  // NS = 2 keeps the data's hi halves only
                        *reinterpret_cast<uint32_t *>(bop + cslot(c) * COMP + off) =
                            pick4(w[c][0], w[c][1], w[c][2], w[c][3], j);
            }
        }
        }
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
        __syncthreads();
        // ---- step 3: D[k1][k2] -----------------------------------------------------
        // the next item's input (the current one again after the last, so that the
        // registers are always reloaded and stay free from the input stage to here)
        const int64_t next = item + gridDim.x < a.n_items ? item + gridDim.x : item;
        if (tid == 0) gemm(KS3, true);
        if (warp != 0) load_input(next);  // lands during the GEMM
        wait_done();
        if (warp == 0) load_input(next);  // not beside the issuing lane
        // ---- output --------------------------------------------------------------
        const float inv = (1.f / s1) * (1.f / s2);  // powers of two: exact
        if (OVL) {
            y_prev = y;
            inv_prev = inv;
        } else {
            store_out(y, inv);
        }
        if (tid == 0 && err) s_err = 1;
        __syncthreads();  // TMEM read out before the next item's MMAs
        if (s_err) break;
    }
    if (OVL && y_prev && !s_err) store_out(y_prev, inv_prev);
    if (s_err && tid == 0) {  // a wait timed out: record it, let copies and MMAs in flight finish (bounded)
        *reinterpret_cast<volatile int *>(a.status) = 1;
        for (int b = 0; b < NRING; ++b)
            if (pend & (1u << b)) mbar_wait(&full[b], (pend_g[b] / NRING) & 1u);
        mma_commit(&done);
        mbar_wait(&done, done_n & 1u);
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tb), "r"(kTmemCols));
}

// ---- CUDA-core steps around the tensor-core transforms ---------------------

// Stage A pairing: packed snapshot -> Z[k], k < 16384 (as k_swarm_c2r).
__global__ void k_tc_prep_a(const uint32_t *__restrict__ spec, int64_t spec_pol_stride, int64_t snap0, int64_t n_snaps,
                            float2 *__restrict__ z, const float2 *__restrict__ w32768) {
    const int64_t item = blockIdx.x;  // pol * n_snaps + s
    const int64_t pol = item / n_snaps, s = item % n_snaps;
    const uint32_t *sp = spec + pol * spec_pol_stride + (snap0 + s) * kGroups;
    float2 *zo = z + item * kMA;
    for (int k = threadIdx.x; k <= kMA / 2; k += blockDim.x) {
        float2 va = nib_value(sp, k);
        float2 vb = make_float2(0.f, 0.f);
        if (k == 0)
            va.y = 0.f;
        else
            vb = nib_value(sp, kMA - k);
        float2 zk, zmk;
        c2r_pair(va, vb, conjf2(__ldg(w32768 + k)), zk, zmk);
        zo[k] = zk;
        if (k != 0 && k != kMA / 2) zo[kMA - k] = zmk;
    }
}

// R2C bin q of a 36608-sample chunk from its half-length transform Z.
__device__ __forceinline__ float2 r2c_at(const float2 *zb, int q, const float2 *w36608) {
    if (q == 0) return make_float2(zb[0].x + zb[0].y, 0.f);
    if (q == kMB) return make_float2(zb[0].x - zb[0].y, 0.f);
    float2 xq, xmq;
    r2c_pair(zb[q], zb[kMB - q], __ldg(w36608 + q), xq, xmq);
    return xq;
}

// Stage B -> C: the R2C pairing of Z (18304 per chunk) and the C2R pairing of
// the bins [skip, skip + 16384] -> Z' (16384 per chunk), as k_resample does.
__global__ void k_tc_pair_bc(const float2 *__restrict__ zb, float2 *__restrict__ zc, int skip,
                             const float2 *__restrict__ w32768, const float2 *__restrict__ w36608) {
    const int64_t item = blockIdx.x;
    const float2 *zi = zb + item * kMB;
    float2 *zo = zc + item * kMA;
    for (int j = threadIdx.x; j <= kMA / 2; j += blockDim.x) {
        float2 yv = r2c_at(zi, skip + j, w36608), ym = r2c_at(zi, skip + kMA - j, w36608);
        if (j == 0) {
            yv.y = 0.f;
            ym.y = 0.f;
        }
        float2 zk, zmk;
        c2r_pair(yv, ym, conjf2(__ldg(w32768 + j)), zk, zmk);
        zo[j] = zk;
        if (j != 0 && j != kMA / 2) zo[kMA - j] = zmk;
    }
}

// C2R pairing of complex spectra X[0..16384] (row stride spec_stride): Z[j],
// Z[16384 - j] from X[j], X[16384 - j], the imaginary parts of X[0] and
// X[16384] dropped (as k_r2dbe_c2r with skip 0).
__global__ void k_tc_pair_c2r(const float2 *__restrict__ spec, int64_t spec_stride, float2 *__restrict__ z,
                              const float2 *__restrict__ w32768) {
    const int64_t item = blockIdx.x;
    const float2 *sp = spec + item * spec_stride;
    float2 *zo = z + item * kMA;
    for (int j = threadIdx.x; j <= kMA / 2; j += blockDim.x) {
        float2 y = sp[j], ym = sp[kMA - j];
        if (j == 0) {
            y.y = 0.f;
            ym.y = 0.f;
        }
        float2 zk, zmk;
        c2r_pair(y, ym, conjf2(__ldg(w32768 + j)), zk, zmk);
        zo[j] = zk;
        if (j != 0 && j != kMA / 2) zo[kMA - j] = zmk;
    }
}

// Per-chunk (n, mean, M2) of the first batch's floats in FP64 (as k_resample<1>).
__global__ void k_tc_chunk_stats(const float *__restrict__ y, int64_t y_pol_stride, int n_chunks,
                                 double *__restrict__ partials) {
    __shared__ double red[64];
    const int pol = blockIdx.y, c = blockIdx.x;
    const float *src = y + pol * y_pol_stride + static_cast<int64_t>(c) * kNC;
    double s1 = 0.0, s2 = 0.0;
    for (int i = threadIdx.x; i < kNC; i += blockDim.x) {
        const double v = src[i];
        s1 += v;
        s2 += v * v;
    }
    block_sum2(s1, s2, red);
    if (threadIdx.x == 0) {
        const double n = static_cast<double>(kNC), mean = s1 / n;
        double *pp = partials + (static_cast<int64_t>(pol) * n_chunks + c) * 3;
        pp[0] = n;
        pp[1] = mean;
        pp[2] = s2 - s1 * mean;
    }
}

// Pre-tiled DFT matrices for the tensor cores: K-step s, component c (re hi,
// re lo, im hi, im lo) holds F[r][16 s + kk], r < rows, kk < 16, in
// core-matrix order (8 rows x 16 bytes; K step 128 bytes, row-group step 256
// bytes); F[m][k] = e^{-2 pi i m k / nf}, zero outside nf x nf.  Layout
// [s][c][rows x 16]: one K-step's tiles are contiguous.
std::vector<__half> dft_tiles(int nf, int rows, int ksteps) {
    std::vector<__half> out(static_cast<size_t>(ksteps) * 4 * rows * 16);
    for (int s = 0; s < ksteps; ++s)
        for (int r = 0; r < rows; ++r)
            for (int kk = 0; kk < 16; ++kk) {
                const int k = 16 * s + kk;
                double re = 0.0, im = 0.0;
                if (r < nf && k < nf) {
                    const long long e = static_cast<long long>(r) * k % nf;
                    const double ang = -2.0 * 3.14159265358979323846 * static_cast<double>(e) / nf;
                    re = std::cos(ang);
                    im = std::sin(ang);
                }
                const float rh = __half2float(__float2half_rn(static_cast<float>(re)));
                const float ih = __half2float(__float2half_rn(static_cast<float>(im)));
                const __half vals[4] = {__float2half_rn(static_cast<float>(re)),
                                        __float2half_rn(static_cast<float>(re - rh)),
                                        __float2half_rn(static_cast<float>(im)),
                                        __float2half_rn(static_cast<float>(im - ih))};
                const size_t off = (r >> 3) * 128 + (kk >> 3) * 64 + (r & 7) * 8 + (kk & 7);  // in halves
                for (int c = 0; c < 4; ++c) out[(static_cast<size_t>(s) * 4 + c) * rows * 16 + off] = vals[c];
            }
    return out;
}

template <int N2, bool INV, int NS>
cudaError_t launch_tc_fft_ns(const TcFftArgs &args, cudaStream_t st) {
    int dev = 0, sms = 1;
    cudaError_t e = cudaGetDevice(&dev);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (e == cudaSuccess)  // cheap; set each time so that every device gets it
        e = cudaFuncSetAttribute(k_tc_fft<N2, INV, NS>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 static_cast<int>(TcGeo<N2, NS>::SMEM));
    if (e != cudaSuccess) return e;
    const unsigned grid = static_cast<unsigned>(args.n_items < sms ? args.n_items : sms);
    k_tc_fft<N2, INV, NS><<<grid, kTcThreads, TcGeo<N2, NS>::SMEM, st>>>(args);
    return cudaGetLastError();
}

// ns = split products per complex product: 3 (SDBE_PRECISION_TC16) or 2 (SDBE_PRECISION_TC16_FAST).
template <int N2, bool INV>
cudaError_t launch_tc_fft(const TcFftArgs &args, int ns, cudaStream_t st) {
    if (args.n_items <= 0) return cudaSuccess;
    return ns == 3 ? launch_tc_fft_ns<N2, INV, 3>(args, st) : launch_tc_fft_ns<N2, INV, 2>(args, st);
}

}  // namespace

// A launch of one segment: n = per_pol items (one pol).
static TcFftArgs one_seg(const TcSeg &g, const uint8_t *f1, const uint8_t *f2, const float2 *tw, int *status) {
    TcFftArgs a{};
    a.n_items = g.per_pol;
    a.n = 1;
    a.s[0] = g;
    a.f1 = f1;
    a.f2 = f2;
    a.tw = tw;
    a.status = status;
    return a;
}

static int tc_splits(const sdbe_resampler *h) { return h->cfg.precision == SDBE_PRECISION_TC16 ? 3 : 2; }

// Tables and scratch of the tensor-core path, on first use.
int tc_prepare(sdbe_resampler *h, cudaStream_t st) {
    if (h->tc_f128) return SDBE_OK;
    const std::vector<__half> f128 = dft_tiles(128, 128, 8), f143 = dft_tiles(143, 144, 9);
    const size_t wave_snaps = static_cast<size_t>(h->wave) * kBatchSnaps;
    const size_t wave_chunks = static_cast<size_t>(h->wave) * kChunks;
    if (cudaMalloc(&h->tc_f128, f128.size() * sizeof(__half)) != cudaSuccess ||
        cudaMalloc(&h->tc_f143, f143.size() * sizeof(__half)) != cudaSuccess ||
        cudaMalloc(&h->tc_bufx, 2 * wave_snaps * kMA * sizeof(float2)) != cudaSuccess ||
        cudaMalloc(&h->tc_bufy, 2 * wave_chunks * kMB * sizeof(float2)) != cudaSuccess ||
        cudaHostAlloc(&h->tc_status_host, sizeof(int), cudaHostAllocMapped) != cudaSuccess) {
        cudaGetLastError();
        return fail(h, SDBE_ERR_NOMEM, "cannot allocate the tensor-core scratch");
    }
    SDBE_CK(h, cudaMemcpyAsync(h->tc_f128, f128.data(), f128.size() * sizeof(__half), cudaMemcpyHostToDevice, st));
    SDBE_CK(h, cudaMemcpyAsync(h->tc_f143, f143.data(), f143.size() * sizeof(__half), cudaMemcpyHostToDevice, st));
    *h->tc_status_host = 0;
    SDBE_CK(h, cudaHostGetDevicePointer(reinterpret_cast<void **>(&h->tc_status), h->tc_status_host, 0));
    SDBE_CK(h, cudaStreamSynchronize(st));  // the host tables are freed on return
    return SDBE_OK;
}

// One wave of the tensor-core chain over several handles (one stream pair
// each): per handle the stage-A pairing, then one launch of each transform
// covering every handle's items (stage A inverse 16384, stage B forward 18304,
// stage C inverse 16384) with the B->C pairing per handle in between, then per
// handle the 2-bit packing into its payload.  With `first` each item is its
// handle's first batch (nb = 1): its FP64 statistics set the thresholds
// before it is packed, as the FP32 path does.
int tc_wave_multi(const std::vector<TcWaveItem> &w, bool first, cudaStream_t st) {
    if (w.empty()) return SDBE_OK;
    sdbe_resampler *h0 = w[0].h;
    if (tc_splits(h0) == 2) return tcf_wave_multi(w, first, st);  // SDBE_PRECISION_TC16_FAST (k_tcf.cu)
    for (const auto &it : w) {
        if (int rc = tc_prepare(it.h, st)) return rc;
        if (*reinterpret_cast<volatile int *>(it.h->tc_status_host))  // written by an earlier call's kernels
            return fail(it.h, SDBE_ERR_CUDA, "a tensor-core transform timed out on its mbarrier wait");
    }
    const Twiddles &tw = h0->tw;
    const uint8_t *f128 = static_cast<const uint8_t *>(h0->tc_f128);
    const uint8_t *f143 = static_cast<const uint8_t *>(h0->tc_f143);
    TcFftArgs A{}, B{}, C{};
    for (TcFftArgs *x : {&A, &B, &C}) {
        x->f1 = f128;
        x->f2 = x == &B ? f143 : f128;
        x->tw = x == &B ? tw.w18304 : tw.w16384;
        x->status = h0->tc_status;
    }
    int64_t units_a = 0, units_bc = 0;
    for (const auto &it : w) {
        sdbe_resampler *h = it.h;
        const int64_t snaps = it.nb * kBatchSnaps, chunks = it.nb * kChunks;
        float2 *ts = reinterpret_cast<float2 *>(h->ts);
        A.s[A.n++] = TcSeg{h->tc_bufx, kMA, snaps * kMA, ts, kMA, h->ts_pol_stride / 2, snaps, A.n_items};
        A.n_items += 2 * snaps;
        B.s[B.n++] = TcSeg{ts, kMB, h->ts_pol_stride / 2, h->tc_bufy, kMB, chunks * kMB, chunks, B.n_items};
        B.n_items += 2 * chunks;
        C.s[C.n++] = TcSeg{h->tc_bufx, kMA, chunks * kMA, h->tc_bufy, kMA, chunks * kMA, chunks, C.n_items};
        C.n_items += 2 * chunks;
        units_a += 2 * snaps;
        units_bc += 2 * chunks;
    }
    const int ns = tc_splits(h0);
    size_t slot = 0;
    if (!first) SDBE_CK(h0, timed_begin(h0, 0, units_a, st, &slot));
    for (const auto &it : w) {  // stage A pairing: packed spectra -> Z (bufx)
        const int64_t snaps = it.nb * kBatchSnaps;
        k_tc_prep_a<<<static_cast<unsigned>(2 * snaps), 256, 0, st>>>(it.spec, it.spec_pol_stride,
                                                                      it.b0 * kBatchSnaps, snaps, it.h->tc_bufx,
                                                                      tw.w32768);
        SDBE_CK(it.h, cudaGetLastError());
    }
    SDBE_CK(h0, (launch_tc_fft<128, true>(A, ns, st)));  // -> time series (ts)
    if (!first) {
        SDBE_CK(h0, timed_end(h0, slot, st));
        SDBE_CK(h0, timed_begin(h0, 1, units_bc, st, &slot));
    }
    SDBE_CK(h0, (launch_tc_fft<143, false>(B, ns, st)));  // chunks of 18304 -> Z (bufy)
    for (const auto &it : w) {  // pairings: bufy -> Z' (bufx)
        k_tc_pair_bc<<<static_cast<unsigned>(2 * it.nb * kChunks), 256, 0, st>>>(it.h->tc_bufy, it.h->tc_bufx,
                                                                                it.h->skip, tw.w32768, tw.w36608);
        SDBE_CK(it.h, cudaGetLastError());
    }
    SDBE_CK(h0, (launch_tc_fft<128, true>(C, ns, st)));  // -> floats (bufy, 32768 per chunk)
    WinUpds U{};
    for (const auto &it : w) {
        sdbe_resampler *h = it.h;
        const int64_t chunks = it.nb * kChunks;
        const float *yf = reinterpret_cast<const float *>(h->tc_bufy);
        const bool win = h->cfg.threshold_mode == SDBE_THRESH_WINDOW;
        if (first) {
            k_tc_chunk_stats<<<dim3(kChunks, 2), 256, 0, st>>>(yf, chunks * kNC, kChunks, h->partials);
            SDBE_CK(h, cudaGetLastError());
            SDBE_CK(h, launch_finalize_thresholds(h->partials, kChunks, h->cfg.pol1_uses_pol0_threshold, h->thr, st));
            h->thresholds_set = true;
            h->launches += 2;
        }
        const PayloadTarget &t = it.tgt;
        SDBE_CK(h, launch_quantize_chunks(yf, chunks * kNC, chunks, h->thr, t.base, t.pol_stride, t.pkt_stride,
                                          t.payload_off, it.b0 * kChunks, st));
        h->launches += 3;  // pairing A, pairing BC, packing
        if (first) h->stream_batch = 0;
        if (win && !first) {  // windowed thresholds: this wave's FP64 chunk statistics
            k_tc_chunk_stats<<<dim3(static_cast<unsigned>(chunks), 2), 256, 0, st>>>(yf, chunks * kNC,
                                                                                  static_cast<int>(chunks), h->wpart);
            SDBE_CK(h, cudaGetLastError());
            h->launches += 1;
        }
        // the window ring takes the wave's statistics after it was packed with the old thresholds
        window_step(h, first ? h->partials : h->wpart, it.nb, true, U);
    }
    if (U.n) {
        SDBE_CK(h0, launch_window_update(U, st));
        h0->launches += 1;
    }
    if (!first) SDBE_CK(h0, timed_end(h0, slot, st));
    h0->launches += 3;  // the three transforms
    return SDBE_OK;
}

// The FFT chain of sdbe_process in the tensor-core form: the first batch of a
// stream alone (it sets the thresholds), then waves of up to `wave` batches.
int tc_chain(sdbe_resampler *h, const uint32_t *spec, int64_t spec_pol_stride, int64_t n_batches,
             const PayloadTarget &tgt, cudaStream_t st, const std::function<int(int64_t, int64_t)> &on_wave) {
    for (int64_t b = 0; b < n_batches;) {
        const bool first = !h->thresholds_set;
        const int64_t nb = first ? 1 : wave_len(h, h->wave, n_batches - b);
        if (int rc = tc_wave_multi({TcWaveItem{h, spec, spec_pol_stride, b, nb, tgt}}, first, st)) return rc;
        if (int rc = on_wave(b * kChunks, (b + nb) * kChunks)) return rc;
        b += nb;
    }
    return SDBE_OK;
}

// Stage entry points in the tensor-core form (sdbe_swarm_c2r and
// sdbe_resample_chunks on a SDBE_PRECISION_TC16 handle), one pol, in pieces
// that fit the handle's scratch.
int tc_swarm_c2r(sdbe_resampler *h, const uint32_t *spec, int64_t n_snaps, float *out, cudaStream_t st) {
    if (n_snaps <= 0) return SDBE_OK;
    if (reinterpret_cast<uintptr_t>(out) & 15u)  // the transform writes 16-byte pieces
        return fail(h, SDBE_ERR_ARG, "SDBE_PRECISION_TC16 needs a 16-byte aligned output buffer");
    if (int rc = tc_prepare(h, st)) return rc;
    const uint8_t *f128 = static_cast<const uint8_t *>(h->tc_f128);
    if (tc_splits(h) == 2) {  // SDBE_PRECISION_TC16_FAST: straight from the packed spectra (k_tcf.cu)
        const TcfASeg seg{spec, 0, 0, n_snaps, out, 0};
        return tcf_stage_a(h, &seg, 1, 1, false, st);
    }
    const int64_t cap = 2 * static_cast<int64_t>(h->wave) * kBatchSnaps;
    for (int64_t s0 = 0; s0 < n_snaps; s0 += cap) {
        const int64_t n = n_snaps - s0 < cap ? n_snaps - s0 : cap;
        k_tc_prep_a<<<static_cast<unsigned>(n), 256, 0, st>>>(spec, 0, s0, n, h->tc_bufx, h->tw.w32768);
        SDBE_CK(h, cudaGetLastError());
        const TcFftArgs A = one_seg(TcSeg{h->tc_bufx, kMA, 0, reinterpret_cast<float2 *>(out + s0 * kNA), kMA, 0, n, 0},
                                    f128, f128, h->tw.w16384, h->tc_status);
        SDBE_CK(h, (launch_tc_fft<128, true>(A, tc_splits(h), st)));
    }
    return SDBE_OK;
}

int tc_resample_chunks(sdbe_resampler *h, const float *in, int64_t n_chunks, float *out, cudaStream_t st) {
    if (n_chunks <= 0) return SDBE_OK;
    if ((reinterpret_cast<uintptr_t>(in) & 7u) || (reinterpret_cast<uintptr_t>(out) & 15u))
        return fail(h, SDBE_ERR_ARG, "SDBE_PRECISION_TC16 needs 8-byte aligned input and 16-byte aligned output");
    if (tc_splits(h) == 2) {  // SDBE_PRECISION_TC16_FAST (k_tcf.cu): FP16 copy of the input, stages B and C
        if (int rc = tcf_prepare(h, st)) return rc;
        const int64_t cap = 2 * static_cast<int64_t>(h->wave) * kChunks;
        if (int rc = grow(h, reinterpret_cast<uint8_t **>(&h->tcf_half), &h->tcf_half_bytes, cap * kNB * 2,
                          "the tensor-core FP16 input"))
            return rc;
        if (int rc = grow(h, reinterpret_cast<uint8_t **>(&h->tcf_bins), &h->tcf_bins_bytes, cap * kTcfBinsLen * 4,
                          "the tensor-core bins"))
            return rc;
        for (int64_t c0 = 0; c0 < n_chunks; c0 += cap) {
            const int64_t n = n_chunks - c0 < cap ? n_chunks - c0 : cap;
            SDBE_CK(h, tcf_to_half(in + c0 * kNB, h->tcf_half, n * kNB, st));
            TcfBCSeg b{};
            b.ts = h->tcf_half;
            b.bins = h->tcf_bins;
            b.n_chunks = n;
            b.skip = h->skip;
            b.o.fout = out + c0 * kNC;
            if (int rc = tcf_stage_bc(h, &b, 1, 1, 5, st)) return rc;
        }
        return SDBE_OK;
    }
    if (int rc = tc_prepare(h, st)) return rc;
    const uint8_t *f128 = static_cast<const uint8_t *>(h->tc_f128);
    const uint8_t *f143 = static_cast<const uint8_t *>(h->tc_f143);
    const int64_t cap = 2 * static_cast<int64_t>(h->wave) * kChunks;
    for (int64_t c0 = 0; c0 < n_chunks; c0 += cap) {
        const int64_t n = n_chunks - c0 < cap ? n_chunks - c0 : cap;
        const TcFftArgs B = one_seg(TcSeg{reinterpret_cast<const float2 *>(in + c0 * kNB), kMB, 0, h->tc_bufy, kMB, 0,
                                          n, 0},
                                    f128, f143, h->tw.w18304, h->tc_status);
        SDBE_CK(h, (launch_tc_fft<143, false>(B, tc_splits(h), st)));
        k_tc_pair_bc<<<static_cast<unsigned>(n), 256, 0, st>>>(h->tc_bufy, h->tc_bufx, h->skip, h->tw.w32768,
                                                               h->tw.w36608);
        SDBE_CK(h, cudaGetLastError());
        const TcFftArgs C = one_seg(TcSeg{h->tc_bufx, kMA, 0, reinterpret_cast<float2 *>(out + c0 * kNC), kMA, 0, n, 0},
                                    f128, f128, h->tw.w16384, h->tc_status);
        SDBE_CK(h, (launch_tc_fft<128, true>(C, tc_splits(h), st)));
    }
    return SDBE_OK;
}

// C2R 32768 of n complex spectra [n][spec_stride >= 16385] into out [n][32768]
// floats in the tensor-core form (the inverse PFB's transform); z is caller
// scratch of n x 16384 complex values.
int tc_c2r_spectra(sdbe_resampler *h, const float2 *spec, int64_t spec_stride, int64_t n, float2 *z, float *out,
                   cudaStream_t st) {
    if (n <= 0) return SDBE_OK;
    if (reinterpret_cast<uintptr_t>(out) & 15u)
        return fail(h, SDBE_ERR_ARG, "the tensor-core precisions need a 16-byte aligned output buffer");
    if (int rc = tc_prepare(h, st)) return rc;
    const uint8_t *f128 = static_cast<const uint8_t *>(h->tc_f128);
    for (int64_t i0 = 0; i0 < n; i0 += (int64_t(1) << 30)) {  // grid limit of the pairing kernel
        const int64_t m = n - i0 < (int64_t(1) << 30) ? n - i0 : (int64_t(1) << 30);
        k_tc_pair_c2r<<<static_cast<unsigned>(m), 256, 0, st>>>(spec + i0 * spec_stride, spec_stride, z + i0 * kMA,
                                                               h->tw.w32768);
        SDBE_CK(h, cudaGetLastError());
    }
    const TcFftArgs A =
        one_seg(TcSeg{z, kMA, 0, reinterpret_cast<float2 *>(out), kMA, 0, n, 0}, f128, f128, h->tw.w16384, h->tc_status);
    SDBE_CK(h, (launch_tc_fft<128, true>(A, tc_splits(h), st)));
    return SDBE_OK;
}

}  // namespace sdbe
