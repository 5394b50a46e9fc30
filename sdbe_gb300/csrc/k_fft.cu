// Resampling FFT kernels: one transform per CTA at a time, the whole transform
// resident in shared memory, persistent grids (one CTA per SM looping over
// transforms, twiddle tables loaded into shared memory once per CTA).
//
// Reference: the three cuFFT plans of vdif_inout_gpu_thread.cu:271-333 run by
// SwarmC2R / SwarmR2C / R2dbeC2R (:589-709) on each 143-snapshot batch.
//   stage A  C2R 32768 per snapshot  = 16384-point complex inverse FFT plus
//            Hermitian pre-processing, fed straight from the packed 2-bit
//            spectrum (beng_int8_to_cufftComplex and the Nyquist memset fused);
//            the next snapshot's 8 KB are prefetched with cp.async.
//   stage BC R2C 36608 per chunk = 18304-point complex FFT + post-processing,
//            bins [skip, skip+16384] selected in registers, C2R 32768 through
//            a 16384-point inverse FFT, then quantize2bit in the epilogue.
// All scaling is cuFFT's unnormalised convention.
#include <cmath>
#include <vector>

#include "fft_core.cuh"
#include "launchers.cuh"
#include "sdbe_internal.cuh"

namespace sdbe {

constexpr int kNTA = 512;   // stage A threads: 512 radix-32 butterflies per pass
constexpr int kNTB = 512;   // stage BC threads: 4 warps per SM sub-partition -> 128 registers
// The 18304-point data (stage BC) is padded one float2 per 16, so that the
// first pass's digit-reversed stores, 16 lanes at a time, land in 16
// distinct bank pairs (see fft18304_from_global); the 16384-point transforms
// keep one per 32 (their layouts are built on it).
__host__ __device__ constexpr int padb(int a) { return a + (a >> 4); }
constexpr int kPadA = padded_len(kMA);
constexpr int kPadB = padb(kMB) + 1;

// Shared-memory twiddle tables (float2).  The per-pass tables are laid out
// [r][k] so that the 16 lanes of a half-warp, which hold consecutive k, read
// consecutive words; the two-level tables are padded with tp().
constexpr int kT32 = 10 * 32;          // W_1024^{j s}, s = 1..7, then W_1024^{8 j a}, a = 1..3 (16384-point pass 2)
constexpr int kT128 = tp_len(128);     // two-level halves
constexpr int kT13 = 12 * 16;          // W_208^{k r}, r = 1..12, k = 0..15   (18304-point radix-13 pass)
constexpr int kH18304 = tp_len(143);   // W_18304^{128 a}
constexpr int kTwA = kT32 + 2 * kT128;               // stage A tables
constexpr int kTwB = kTwA + kT13 + kH18304 + kT128;  // stage BC tables
constexpr size_t kSmemA = 2 * kGroups * sizeof(uint32_t) + (kPadA + kTwA) * sizeof(float2);
constexpr size_t kSmemB = (kPadB + kTwB) * sizeof(float2);
// Stage BC fits the 164 KB shared-memory carveout (with its 512-byte static
// reduction buffer and the 1 KB reserved per block).  Above it (184 KB: the
// 196 KB carveout) the kernel measured 1% slower, even with a radix-11
// twiddle table that saves work, and at 208 KB (the 228 KB carveout) 9.5%
// slower.
static_assert(kSmemB + 512 + 1024 <= 164 * 1024, "stage BC shared memory above the 164 KB carveout");

// ---- table loading --------------------------------------------------------
struct TabsA {  // inverse-16384 tables
    float2 *t32, *h16384, *l16384;
};
struct TabsB {  // forward-18304 tables in shared memory; W_36608^q in global memory
    float2 *t13, *h18304, *l18304;
    const float2 *w36608;
};

__device__ __forceinline__ TabsA tabs_a_at(float2 *p) {
    return TabsA{p, p + kT32, p + kT32 + kT128};
}

__device__ __forceinline__ void load_tabs_a(TabsA t, const Twiddles &tw) {
    for (int m = threadIdx.x; m < kT32; m += blockDim.x) {
        const int j = m & 31, g = m >> 5;                       // g < 7: s = g + 1; else a = g - 6
        const int e = g < 7 ? j * (g + 1) : 8 * j * (g - 6);   // exponent of W_1024
        t.t32[m] = __ldg(tw.w16384 + 16 * e);
    }
    for (int m = threadIdx.x; m < 128; m += blockDim.x) {
        t.h16384[tp(m)] = __ldg(tw.w16384 + 128 * m);
        t.l16384[tp(m)] = __ldg(tw.w16384 + m);
    }
}

__device__ __forceinline__ void load_tabs_b(TabsB t, const Twiddles &tw) {
    for (int m = threadIdx.x; m < kT13; m += blockDim.x) {
        const int r = (m >> 4) + 1, k = m & 15;
        t.t13[m] = __ldg(tw.w18304 + 88 * k * r);
    }
    for (int m = threadIdx.x; m < 143; m += blockDim.x) t.h18304[tp(m)] = __ldg(tw.w18304 + 128 * m);
    for (int m = threadIdx.x; m < 128; m += blockDim.x) t.l18304[tp(m)] = __ldg(tw.w18304 + m);
}

__device__ __forceinline__ TabsB tabs_b_at(float2 *tb, const Twiddles &tw) {
    float2 *p = tb + kTwA;
    return TabsB{p, p + kT13, p + kT13 + kH18304, tw.w36608};
}

// First-pass lane order of the 18304-point transform: half-warp h takes the
// groups of 8 consecutive inputs g0 = kFirstPassGroups[2h], g1 = [2h+1]
// (inputs j = 8g + c, c = 0..7; 255 = none).  Output slot 16*rho(j) + r has
// rho(8g + c) = rho(8g) - c (mod 16); the pairs are chosen with rho(8 g1) =
// rho(8 g0) + 8 (mod 16), so the 16 lanes' padded slots cover all 16 bank
// pairs and every store is one wavefront.
__constant__ uint8_t kFirstPassGroups[144] = {
    0,   8,   28,  14,  34,  42,  62,  48,  68,  76,  96,  82,  102, 88,  130, 116, 136, 122, 5,   19,  11,  25,
    39,  53,  45,  59,  73,  87,  79,  93,  107, 99,  113, 127, 141, 133, 10,  2,   16,  30,  22,  36,  50,  64,
    56,  70,  84,  98,  90,  104, 118, 110, 124, 138, 21,  7,   27,  13,  33,  41,  61,  47,  67,  75,  95,  81,
    101, 109, 129, 115, 135, 121, 4,   18,  32,  24,  38,  52,  44,  58,  72,  86,  78,  92,  106, 120, 112, 126,
    140, 132, 9,   1,   15,  29,  43,  35,  49,  63,  55,  69,  83,  97,  89,  103, 117, 131, 123, 137, 20,  6,
    26,  12,  54,  40,  60,  46,  66,  74,  94,  80,  100, 108, 128, 114, 134, 142, 3,   17,  31,  23,  37,  51,
    65,  57,  71,  85,  77,  91,  105, 119, 111, 125, 139, 255};

// ---------------------------------------------------------------------------
// Inverse 16384-point FFT, radices 32 x 32 x 16 (Stockham).  zin(v) gives
// input elements col + 512 r, r < 32, of this thread's first-pass column
// `col` (a permutation of the thread index whose 16 values in each half-warp
// are distinct mod 16; zin may read `sm`: a barrier separates those reads
// from the writes); epi(jj, u) receives outputs z[jj + 1024 r], r < 16.
// blockDim.x is 512.
// The last pass's per-thread twiddle bases W_16384^(tid s), s = 1..3, and
// W_16384^(4 tid a), a = 1..3: they depend on the thread only, so a
// persistent kernel can form them once.
struct LastTw {
    float2 S0[4], A0[4];
};
__device__ __forceinline__ LastTw last_tw(const TabsA &T) {
    LastTw t;
    const int tid = threadIdx.x;
#pragma unroll
    for (int s = 1; s < 4; ++s) t.S0[s] = tw2(T.h16384, T.l16384, tid * s);
#pragma unroll
    for (int a = 1; a < 4; ++a) t.A0[a] = tw2(T.h16384, T.l16384, tid * 4 * a);
    return t;
}

// ZIN_SM: zin reads `sm`, so a barrier must separate those reads from the
// first pass's stores.  A caller whose zin reads other memory, and whose
// previous smem reads are behind a barrier already, passes false.
template <bool ZIN_SM = true, class In, class Epi>
__device__ __forceinline__ void ifft16384(float2 *sm, const TabsA &T, In zin, Epi epi, int col, const LastTw &lt) {
    const int tid = threadIdx.x;
    float2 v[32];
    if (tid < 512) {
        zin(v);
        dft<32, true>(v);
    }
    if constexpr (ZIN_SM) __syncthreads();
    // padded addresses as base + compile-time offsets: pad(32 t + r) = 33 t + r,
    // pad(t + 512 r) = pad(t) + 528 r, pad(b + 32 r) = pad(b) + 33 r (b % 32 + r < 32 not
    // needed: b is a multiple of 1024 plus a lane), pad(j + 1024 r) = pad(j) + 1056 r.
    if (tid < 512) {
        float2 *dst = sm + 33 * col;
#pragma unroll
        for (int r = 0; r < 32; ++r) dst[r] = v[r];
    }
    __syncthreads();
    if (tid < 512) {
        const float2 *src = sm + pad(tid);
#pragma unroll
        for (int r = 0; r < 32; ++r) v[r] = src[528 * r];
        // W_1024^{jm r} = A[r/8] * S[r%8]
        const float2 *tj = T.t32 + (tid & 31);
        float2 S[8], A[4];
#pragma unroll
        for (int s = 1; s < 8; ++s) S[s] = tj[32 * (s - 1)];
#pragma unroll
        for (int a = 1; a < 4; ++a) A[a] = tj[32 * (6 + a)];
#pragma unroll
        for (int r = 1; r < 32; ++r) {
            const int a = r >> 3, s = r & 7;
            const float2 w = a == 0 ? S[s] : (s == 0 ? A[a] : cmul(A[a], S[s]));
            v[r] = cmulc(v[r], w);
        }
        dft<32, true>(v);
    }
    __syncthreads();
    if (tid < 512) {
        float2 *dst = sm + (tid >> 5) * 1056 + (tid & 31);
#pragma unroll
        for (int r = 0; r < 32; ++r) dst[33 * r] = v[r];
    }
    __syncthreads();
    // last pass: jj = tid + 512 i, i = 0, 1; W_16384^(jj s) = W^(tid s) W^(512 i s)
    const float2 *S0 = lt.S0, *A0 = lt.A0;
#pragma unroll
    for (int i = 0; i < 2; ++i) {
        const int jj = tid + 512 * i;
        float2 u[16];
        const float2 *src = sm + pad(jj);
#pragma unroll
        for (int r = 0; r < 16; ++r) u[r] = src[1056 * r];
        // W_16384^{jj r} = A[r/4] * S[r%4]
        float2 S[4], A[4];
        S[1] = i ? mul_tc<kMA, 512, false>(S0[1]) : S0[1];
        S[2] = i ? mul_tc<kMA, 1024, false>(S0[2]) : S0[2];
        S[3] = i ? mul_tc<kMA, 1536, false>(S0[3]) : S0[3];
        A[1] = i ? mul_tc<kMA, 2048, false>(A0[1]) : A0[1];
        A[2] = i ? mul_tc<kMA, 4096, false>(A0[2]) : A0[2];
        A[3] = i ? mul_tc<kMA, 6144, false>(A0[3]) : A0[3];
#pragma unroll
        for (int r = 1; r < 16; ++r) {
            const int a = r >> 2, s = r & 3;
            const float2 w = a == 0 ? S[s] : (s == 0 ? A[a] : cmul(A[a], S[s]));
            u[r] = cmulc(u[r], w);
        }
        dft<16, true>(u);
        epi(jj, u);
    }
}

// The same, forming the last pass's twiddle bases on each call (for kernels
// with no registers to keep them across items).
template <class In, class Epi>
__device__ __forceinline__ void ifft16384(float2 *sm, const TabsA &T, In zin, Epi epi, int col = threadIdx.x) {
    ifft16384(sm, T, zin, epi, col, last_tw(T));
}

// f(integral_constant<int, R>) for each R: a loop over compile-time indices.
template <int... R, class F>
__device__ __forceinline__ void for_r(std::integer_sequence<int, R...>, F f) {
    (f(std::integral_constant<int, R>{}), ...);
}

// Forward 18304-point FFT of z[m] = x[2m] + i x[2m+1] read from global memory;
// result Z in natural order in `sm` (padded with padb).  In-place decimation
// in time, radices 16 (from global) x 13 x 11 x 8: the first pass reads
// z[j + 1144 r] (8 consecutive j per 8 lanes: 64-B segments) and writes its 16
// outputs to slots 16*rho(j) + r, rho = digit reversal of j over (8, 11, 13);
// every later butterfly reads and writes the same slots g*Ns*R + k + Ns*r
// with twiddles W_{Ns*R}^{k r}, so passes need no staging.
//
// R2C: the last pass also applies the R2C pairing, leaving X[q] (q <= 18304,
// X[18304] in the spare slot padb(18304)) instead of Z.  Its butterfly k
// holds Z[k + 2288 r] and butterfly 2288 - k holds their mirrors Z[18304 - q]
// at r' = 7 - r, so one thread takes both (k = 0 and k = 1144 are their own
// mirrors) and pairs in registers: one pass and one barrier fewer.
template <bool R2C>
__device__ __forceinline__ void fft18304_from_global(float2 *sm, const float2 *__restrict__ z, const TabsB &T) {
    constexpr int NB1 = kMB / 16;  // 1144 = 143 groups of 8
    for (int h = threadIdx.x >> 4; h < 72; h += blockDim.x >> 4) {
        const int g = kFirstPassGroups[2 * h + ((threadIdx.x >> 3) & 1)];
        if (g == 255) continue;
        const int c = threadIdx.x & 7, j = 8 * g + c;
        float2 v[16];
        // read-only loads (ld.global.nc), not streaming ones (ld.global.cs):
        // measured 2% faster for the kernel, though L1 hits stay rare (7% of
        // sectors), so the gain is not from reuse of the other half of each
        // 128-byte line
#pragma unroll
        for (int r = 0; r < 16; ++r) v[r] = __ldg(z + j + NB1 * r);
        dft<16, false>(v);
        // rho(8g + c) = g/11 + 13 (g%11) + 143 c; padb(16 rho + r) = 17 rho + r (r < 16)
        float2 *d = sm + 17 * (g / 11 + 13 * (g % 11) + 143 * c);
#pragma unroll
        for (int r = 0; r < 16; ++r) d[r] = v[r];
    }
    __syncthreads();
    // radix 13, Ns = 16: twiddles W_208^{k r}; k = b & 15 = tid & 15 for all of a
    // thread's butterflies (blockDim.x is a multiple of 16), so they load once
    {
        const int k = threadIdx.x & 15;
        float2 w13[13];
#pragma unroll
        for (int r = 1; r < 13; ++r) w13[r] = T.t13[16 * (r - 1) + k];
        for (int b = threadIdx.x; b < kMB / 13; b += blockDim.x) {
            float2 *p = sm + padb((b >> 4) * 208 + k);  // padb(base + 16 r) = padb(base) + 17 r
            float2 v[13];
#pragma unroll
            for (int r = 0; r < 13; ++r) v[r] = p[17 * r];
#pragma unroll
            for (int r = 1; r < 13; ++r) v[r] = cmul(v[r], w13[r]);
            dft<13, false>(v);
#pragma unroll
            for (int r = 0; r < 13; ++r) p[17 * r] = v[r];
        }
    }
    __syncthreads();
    // radix 11, Ns = 208: twiddles W_2288^{k r}.  Butterfly (m, k) is at base
    // 2288 m + k, m < 8, k < 208; thread t takes k = t % 208 and m = t / 208
    // + j nk, nk = the threads sharing its k, so its ten twiddles are formed
    // once per transform, from the two-level W_18304 tables (at most 4
    // butterflies a thread, as with b = t + 512 j).
    {
        static_assert(kNTB == 512, "512 threads share 208 x 8 butterflies");
        const int t = threadIdx.x, k = t % 208, nk = k < 512 - 2 * 208 ? 3 : 2;
        float2 w11[11];
#pragma unroll
        for (int r = 1; r < 11; ++r) w11[r] = tw2(T.h18304, T.l18304, 8 * k * r);  // W_2288^(k r), 8 k r < 18304
        for (int m = t / 208; m < 8; m += nk) {
            float2 *p = sm + padb(2288 * m + k);  // padb(base + 208 r) = padb(base) + 221 r
            float2 v[11];
#pragma unroll
            for (int r = 0; r < 11; ++r) v[r] = p[221 * r];
#pragma unroll
            for (int r = 1; r < 11; ++r) v[r] = cmul(v[r], w11[r]);
            dft<11, false>(v);
#pragma unroll
            for (int r = 0; r < 11; ++r) p[221 * r] = v[r];
        }
    }
    __syncthreads();
    // radix 8, Ns = 2288: twiddles W_18304^{k r} = A[r/4] * S[r%4]
    // butterfly k with its twiddles S[q] = W^(k q), q = 1..3, and A1 = W^(4 k)
    auto bfly8w = [&](int k, float2 *v, const float2 *S, float2 A1) {
        const float2 *p = sm + padb(k);  // padb(k + 2288 r) = padb(k) + 2431 r
#pragma unroll
        for (int r = 0; r < 8; ++r) v[r] = p[2431 * r];
#pragma unroll
        for (int r = 1; r < 8; ++r) {
            const float2 w = r < 4 ? S[r] : (r == 4 ? A1 : cmul(A1, S[r - 4]));
            v[r] = cmul(v[r], w);
        }
        dft<8, false>(v);
    };
    auto bfly8 = [&](int k, float2 *v) {
        float2 S[4];
#pragma unroll
        for (int q = 1; q < 4; ++q) S[q] = tw2(T.h18304, T.l18304, k * q);
        bfly8w(k, v, S, tw2(T.h18304, T.l18304, 4 * k));
    };
    if constexpr (!R2C) {
        for (int k = threadIdx.x; k < kMB / 8; k += blockDim.x) {
            float2 v[8];
            bfly8(k, v);
            float2 *p = sm + padb(k);
#pragma unroll
            for (int r = 0; r < 8; ++r) p[2431 * r] = v[r];
        }
    } else {
        constexpr int K = kMB / 8;  // 2288
        // Units u = tid + 512 i (i < 3, u <= 1144).  Twiddles from per-thread
        // bases and compile-time factors: W_18304^(u q) = W^(tid q) W^(512 i q);
        // the mirror butterfly's W^((2288 - u) q) = W^(2288 q) conj(W^(u q));
        // W_36608^(u + 2288 r) = W_36608^u W_16^r.
        static_assert(kNTB == 512, "units u = tid + 512 i");
        const int tid = threadIdx.x;
        float2 B[5];
#pragma unroll
        for (int q = 1; q <= 4; ++q) B[q] = tw2(T.h18304, T.l18304, tid * q);
        const float2 wt = __ldg(T.w36608 + tid);  // W_36608^tid
        for_r(std::make_integer_sequence<int, 3>{}, [&](auto ic) {
            constexpr int i = decltype(ic)::value;
            const int u = tid + 512 * i;
            if (u > K / 2) return;
            float2 S[4];
            S[1] = mul_tc<kMB, 512 * i, false>(B[1]);
            S[2] = mul_tc<kMB, 1024 * i, false>(B[2]);
            S[3] = mul_tc<kMB, 1536 * i, false>(B[3]);
            const float2 A1 = mul_tc<kMB, 2048 * i, false>(B[4]);
            float2 a[8];
            bfly8w(u, a, S, A1);
            float2 *pa = sm + padb(u);
            const float2 wu = mul_tc<kNB, 512 * i, false>(wt);
            if (u == 0) {  // q = 2288 r pairs with 2288 (8 - r); X[0], X[18304] from Z[0]
                pa[0] = make_float2(a[0].x + a[0].y, 0.f);
                sm[padb(kMB)] = make_float2(a[0].x - a[0].y, 0.f);
                for_r(std::integer_sequence<int, 1, 2, 3, 4>{}, [&](auto rc) {
                    constexpr int r = decltype(rc)::value;
                    float2 xq, xmq;
                    r2c_pair(a[r], a[8 - r], mul_tc<16, r, false>(make_float2(1.f, 0.f)), xq, xmq);
                    pa[2431 * r] = xq;
                    if (r != 4) pa[2431 * (8 - r)] = xmq;
                });
            } else if (u == K / 2) {  // q = 1144 + 2288 r pairs with r' = 7 - r
                for_r(std::make_integer_sequence<int, 4>{}, [&](auto rc) {
                    constexpr int r = decltype(rc)::value;
                    float2 xq, xmq;
                    r2c_pair(a[r], a[7 - r], mul_tc<16, r, false>(wu), xq, xmq);
                    pa[2431 * r] = xq;
                    pa[2431 * (7 - r)] = xmq;
                });
            } else {  // butterflies u and 2288 - u
                float2 Sm[4];
                Sm[1] = mul_tc<kMB, K, false>(conjf2(S[1]));
                Sm[2] = mul_tc<kMB, 2 * K, false>(conjf2(S[2]));
                Sm[3] = mul_tc<kMB, 3 * K, false>(conjf2(S[3]));
                float2 b[8];
                bfly8w(K - u, b, Sm, mul_tc<kMB, 4 * K, false>(conjf2(A1)));
                float2 *pb = sm + padb(K - u);
                for_r(std::make_integer_sequence<int, 8>{}, [&](auto rc) {
                    constexpr int r = decltype(rc)::value;
                    float2 xq, xmq;
                    r2c_pair(a[r], b[7 - r], mul_tc<16, r, false>(wu), xq, xmq);
                    pa[2431 * r] = xq;
                    pb[2431 * (7 - r)] = xmq;
                });
            }
        });
    }
    __syncthreads();
}

// Unnormalised R2C bin q (0 <= q <= 18304) of the 36608 real samples from the
// half-length complex transform Z in `sm`, given w = e^{-2 pi i q/36608}:
//   X[q] = (Z[q] + conj Z[M-q])/2 - i w (Z[q] - conj Z[M-q])/2.
__device__ __forceinline__ float2 r2c_bin(const float2 *sm, int q, float2 w) {
    const int qa = q == kMB ? 0 : q;
    const int qb = q == 0 ? 0 : kMB - q;
    const float2 za = sm[padb(qa)];
    const float2 zb = conjf2(sm[padb(qb)]);
    const float2 s = cadd(za, zb), d = csub(za, zb);
    const float2 wd = cmul(w, d);
    return make_float2(0.5f * (s.x + wd.y), 0.5f * (s.y - wd.x));
}

// Hermitian pre-processing of a C2R of length 32768 from bins Y[0..16384],
// given we = e^{+2 pi i k/32768}:
//   Z[k] = (Y[k] + conj Y[M-k]) + i we (Y[k] - conj Y[M-k]),
// imaginary parts of Y[0] and Y[16384] ignored (as cuFFT / numpy do).
__device__ __forceinline__ float2 c2r_pre(float2 y, float2 ym, int k, float2 we) {
    if (k == 0) {
        y.y = 0.f;
        ym.y = 0.f;
    }
    const float2 e = make_float2(y.x + ym.x, y.y - ym.y);
    const float2 o = cmul(make_float2(y.x - ym.x, y.y + ym.y), we);
    return make_float2(e.x - o.y, e.y + o.x);
}

// e^{+2 pi i (tid + 512 r)/32768} for r = 0..31 from one table value.
template <int R>
__device__ __forceinline__ float2 c2r_tw(float2 base) {
    return mul_tc<64, R, true>(base);
}

// First-pass column of thread t for the paired C2R input below: lanes l < 16
// of warp w take b = 16 w + l, lanes l >= 16 take 512 - (16 w + l - 16), so
// lanes l and l ^ 16 hold mirror columns (b + b' = 512); warp 0's lane 16
// takes 256.  The 16 columns of each half-warp are distinct mod 16.
__device__ __forceinline__ int c2r_col(int t) {
    const int w = t >> 5, l = t & 31;
    if (l < 16) return 16 * w + l;
    return (w == 0 && l == 16) ? 256 : 512 - 16 * w - (l - 16);
}

// The C2R 32768 input Z[col + 512 r], r < 32, from the bins Y[0..16384]
// (M = 16384): Z[k] = (Y[k] + conj Y[M-k]) + i e^{2 pi i k/32768}
// (Y[k] - conj Y[M-k]), Im Y[0] and Im Y[M] dropped (Y[M] = 0 if NYQ_ZERO).
// Each pair (k, M - k) is formed once: for p < 16 the thread pairs its
// k = col + 512 p with M - k, which is element 31 - p of the mirror column
// 512 - col, held by lane l ^ 16; one shuffle swaps the halves.  Columns 0
// and 256 are their own mirrors (M - 512 p = 512 (32 - p); M - 256 - 512 p
// = 256 + 512 (31 - p)) and keep both halves; column 0 forms Z[8192] alone.
// lo(p) = Y[col + 512 p] (p <= 16), hi(p) = Y[M - col - 512 p] (p < 16);
// wcol = e^{2 pi i col/32768}.
template <bool NYQ_ZERO, class Lo, class Hi>
__device__ __forceinline__ void c2r_paired(float2 *v, int col, float2 wcol, Lo lo, Hi hi) {
    const int lane = threadIdx.x & 31;
    auto pairs = [&](auto w0c) {
        constexpr bool W0 = decltype(w0c)::value;
        for_r(std::make_integer_sequence<int, 16>{}, [&](auto pc) {
            constexpr int p = decltype(pc)::value;
            float2 y = lo(pc), ym = hi(pc);
            if (W0 && p == 0 && col == 0) {
                y.y = 0.f;
                ym = NYQ_ZERO ? make_float2(0.f, 0.f) : make_float2(ym.x, 0.f);
            }
            float2 zk, zmk;
            c2r_pair(y, ym, c2r_tw<p>(wcol), zk, zmk);
            v[p] = zk;
            const float2 x = make_float2(__shfl_xor_sync(0xffffffffu, zmk.x, 16), __shfl_xor_sync(0xffffffffu, zmk.y, 16));
            if constexpr (!W0) {
                v[31 - p] = x;
            } else {  // selects, not branches: warp 0 must not fall behind
                const bool own = lane == 16;
                v[31 - p] = make_float2(own ? zmk.x : x.x, own ? zmk.y : x.y);
                if constexpr (p >= 1) {
                    const bool c0 = lane == 0;
                    v[32 - p] = make_float2(c0 ? zmk.x : v[32 - p].x, c0 ? zmk.y : v[32 - p].y);
                }
            }
        });
    };
    if (threadIdx.x >= 32) {
        pairs(std::false_type{});
    } else {
        pairs(std::true_type{});
        // column 0: Z[8192] = Y[8192] + conj Y[8192] + i e^{i pi/2} (Y[8192] - conj Y[8192]);
        // the other lanes' lo(16) is in range and discarded
        const float2 y = lo(std::integral_constant<int, 16>{});
        const float2 z = c2r_pre(y, y, 8192, c2r_tw<16>(wcol));
        const bool c0 = lane == 0;
        v[16] = make_float2(c0 ? z.x : v[16].x, c0 ? z.y : v[16].y);
    }
}


__device__ __forceinline__ void cp_async16(void *smem, const void *gmem) {
    const unsigned s = static_cast<unsigned>(__cvta_generic_to_shared(smem));
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(s), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait_1() { asm volatile("cp.async.wait_group 1;\n" ::: "memory"); }

// ---------------------------------------------------------------------------
// Stage A (persistent): items = n_snaps x n_pols.  Packed spectrum of snapshot
// s of pol p at spec + p*spec_pol_stride + (snap0 + s)*2048; time series to
// out + p*out_pol_stride + s*32768.
template <class Segs>
__device__ __forceinline__ int seg_of(const Segs &S, int64_t item) {
    int j = 0;
    while (j + 1 < S.n && item >= S.s[j + 1].item0) ++j;
    return j;
}

__global__ void __launch_bounds__(kNTA, 1) k_swarm_c2r(const __grid_constant__ SegsA S, Twiddles tw) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    uint32_t *sp = reinterpret_cast<uint32_t *>(smem_raw);  // [2][2048] double buffer
    float2 *sm = reinterpret_cast<float2 *>(smem_raw + 2 * kGroups * sizeof(uint32_t));
    TabsA T = tabs_a_at(sm + kPadA);
    load_tabs_a(T, tw);
    const int col = c2r_col(threadIdx.x);               // the inverse's first-pass column
    const float2 wc = conjf2(__ldg(tw.w32768 + col));  // W_32768^-col
    __syncthreads();                                    // tables loaded
    const LastTw lt = last_tw(T);                       // once per CTA
    const int64_t n_items = S.n_items;
    auto src_of = [&](int64_t item) {
        const SegA &g = S.s[seg_of(S, item)];
        const int64_t local = item - g.item0;
        const int64_t pol = local >= g.n_snaps, s = local - pol * g.n_snaps;  // n_pols <= 2: no division
        return reinterpret_cast<const uint4 *>(g.spec + pol * g.spec_pol_stride + (g.snap0 + s) * kGroups);
    };
    int64_t item = blockIdx.x;
    if (item < n_items) cp_async16(sp + 4 * threadIdx.x, src_of(item) + threadIdx.x);
    cp_async_commit();
    for (int buf = 0; item < n_items; item += gridDim.x, buf ^= 1) {
        const int64_t next = item + gridDim.x;
        if (next < n_items) cp_async16(sp + (buf ^ 1) * kGroups + 4 * threadIdx.x, src_of(next) + threadIdx.x);
        cp_async_commit();
        cp_async_wait_1();
        __syncthreads();  // this item's spectrum landed; tables loaded
        const uint32_t *cur = sp + buf * kGroups;
        const SegA &g = S.s[seg_of(S, item)];
        const int64_t local = item - g.item0;
        const int64_t pol = local >= g.n_snaps, s = local - pol * g.n_snaps;
        float2 *dst = reinterpret_cast<float2 *>(g.out + pol * g.out_pol_stride + s * kNA);
        // The inverse's first pass forms Z[col + 512 r] from the packed bins
        // X[k] (k < 16384; the Nyquist bin X[16384] = 0, Im X[0] dropped), each
        // Hermitian pair once with its mirror half from lane ^ 16: no pairing
        // pass, no barrier of its own.
        auto zin = [&](float2 *v) {
            c2r_paired<true>(
                v, col, wc, [&](auto pc) { return nib_value(cur, col + kNTA * decltype(pc)::value); },
                [&](auto pc) {
                    constexpr int p = decltype(pc)::value;
                    const int k = kMA - col - kNTA * p;  // 16384 only for col = 0, p = 0 (replaced by 0)
                    return nib_value(cur, p == 0 ? (k & (kMA - 1)) : k);
                });
        };
        auto epi = [&](int jj, const float2 *u) {
#pragma unroll
            for (int r = 0; r < 16; ++r) __stcs(dst + jj + 1024 * r, u[r]);
        };
        // zin reads the packed spectrum (`cur`), not `sm`, and the barrier at
        // the top of this loop follows the previous item's last reads of `sm`
        ifft16384<false>(sm, T, zin, epi, col, lt);
    }
}

// ---------------------------------------------------------------------------
// Stage BC (persistent): items = n_chunks x n_pols.  Chunk c of pol p: 36608
// floats at in + p*in_pol_stride + c*36608.
//   MODE 0: quantize with thr[p] / thr[2+p] into the u32 payload at
//           out + p*out_pol_stride + (pkt0 + c)*pkt_stride + payload_off.
//   MODE 1: floats to fout + p*fout_pol_stride + c*32768 and per-chunk
//           (n, mean, M2) in FP64 to partials[(p*n_chunks + c)*3].
//   MODE 2: floats only.
//   MODE 3: MODE 0, plus the (n, sum, sum of squares) of each chunk's
//           floats (FP32 per thread and warp, FP64 across warps) to partials
//           when the segment has them (windowed thresholds).
template <int MODE>
__global__ void __launch_bounds__(kNTB, 1) k_resample(const __grid_constant__ SegsB S, Twiddles tw) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    float2 *sm = reinterpret_cast<float2 *>(smem_raw);
    float2 *tb = sm + kPadB;
    TabsA TA = tabs_a_at(tb);
    TabsB TB = tabs_b_at(tb, tw);
    __shared__ double red[64];
    load_tabs_a(TA, tw);
    load_tabs_b(TB, tw);
    const int tid = threadIdx.x;
    const float2 wc = conjf2(__ldg(tw.w32768 + tid));  // W_32768^-tid
    const int64_t n_items = S.n_items;
    for (int64_t item = blockIdx.x; item < n_items; item += gridDim.x) {
        const SegB &g = S.s[seg_of(S, item)];
        const ResampleOut &o = g.o;
        const int n_chunks = g.n_chunks, skip = g.skip;
        const int64_t local = item - g.item0;
        const int pol = local >= n_chunks;  // n_pols <= 2: no division
        const int64_t c = local - pol * n_chunks;
        __syncthreads();  // tables loaded / previous item's last smem reads done
        const float2 *z = reinterpret_cast<const float2 *>(g.in + pol * g.in_pol_stride + c * kNB);
        // forward 18304 with the R2C pairing in its last pass: X[q], q <= 18304
        fft18304_from_global<true>(sm, z, TB);
        // The next item's 146 KB chunk to L2 while this chunk's inverse runs,
        // as nine bulk prefetches from nine threads: pass 1 of the next
        // forward then reads from L2, not HBM.  Per-thread prefetch
        // instructions (9 per thread) cost about 1k cycles of issue per chunk
        // and gained 0.5%; prefetching at the start of the chunk, or two
        // chunks ahead, gained less.
        if (item + gridDim.x < n_items) {
            const int64_t nx = item + gridDim.x;
            const SegB &gn = S.s[seg_of(S, nx)];
            const int64_t ln = nx - gn.item0;
            const int64_t pn = ln >= gn.n_chunks;
            const char *zn = reinterpret_cast<const char *>(gn.in + pn * gn.in_pol_stride + (ln - pn * gn.n_chunks) * kNB);
            if (tid < 9) {  // 146432 B = 8 x 16384 + 15360, 16-byte aligned pieces
                const uint32_t bytes = tid < 8 ? 16384u : static_cast<uint32_t>(kNB * 4 - 8 * 16384);
                asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;" ::"l"(zn + 16384 * tid), "r"(bytes) : "memory");
            }
        }
        // The inverse's first pass loads Z'[j], j = tid + 512 r, computed on the
        // fly by the C2R pairing of the window Y[j] = X[skip + j], j = 0..16384
        // (no pass of its own; ifft16384 syncs before its first stores), with
        // W_32768^-j = wc e^{2 pi i r/64} (wc per thread, the rest compile-time);
        // Im Y[0] and Im Y[16384] are dropped.
        auto zin = [&](float2 *v) {
            const float2 *lo = sm + padb(skip + tid);        // Y[tid + 512 r] = lo[544 r]
            const float2 *hi = sm + padb(skip + kMA - tid);  // Y[16384 - tid - 512 r] = hi[-544 r]
            for_r(std::make_integer_sequence<int, 32>{}, [&](auto rc) {
                constexpr int r = decltype(rc)::value;
                v[r] = c2r_pre(lo[544 * r], hi[-544 * r], tid + 512 * r, c2r_tw<r>(wc));
            });
        };
        if constexpr (MODE == 0 || MODE == 3) {
            uint32_t *words = reinterpret_cast<uint32_t *>(o.out + pol * o.out_pol_stride +
                                                           (o.pkt0 + c) * o.pkt_stride + o.payload_off);
            const float th = o.thr[pol], off = o.thr[2 + pol];
            float f1 = 0.f, f2 = 0.f;
            // Word (jj >> 3) + 128 r holds the 4-bit codes of outputs jj + 1024 r
            // of the 8 lanes jj & 7 = c (lane c at bits 4c).  Each lane builds
            // its codes of rows r < 8 and 8 <= r < 16 as two words (row r at
            // bits 4 (r % 8)); an 8 x 8 nibble transpose over the 8 lanes then
            // leaves lane c with the output words of rows c and 8 + c.
            auto epi = [&](int jj, const float2 *u) {
                uint32_t wl = 0, wh = 0;
#pragma unroll
                for (int r = 0; r < 8; ++r) {
                    wl |= (code2(u[r].x, th, off) | (code2(u[r].y, th, off) << 2)) << (4 * r);
                    wh |= (code2(u[8 + r].x, th, off) | (code2(u[8 + r].y, th, off) << 2)) << (4 * r);
                }
                if constexpr (MODE == 3) {
#pragma unroll
                    for (int r = 0; r < 16; ++r) {
                        f1 += u[r].x + u[r].y;
                        f2 = fmaf(u[r].x, u[r].x, fmaf(u[r].y, u[r].y, f2));
                    }
                }
                const int c = jj & 7;
                wl = nib_transpose8(wl, c);
                wh = nib_transpose8(wh, c);
                words[(jj >> 3) + 128 * c] = wl;
                words[(jj >> 3) + 128 * (8 + c)] = wh;
            };
            ifft16384(sm, TA, zin, epi);
            if constexpr (MODE == 3) {
                if (o.partials != nullptr) {  // uniform over the block
                    double s1, s2;
                    block_sum2_f(f1, f2, s1, s2, red);
                    if (tid == 0) {
                        double *pp = o.partials + (static_cast<int64_t>(pol) * n_chunks + c) * 3;
                        pp[0] = static_cast<double>(kNC);
                        pp[1] = s1;
                        pp[2] = s2;
                    }
                }
            }
        } else {
            float2 *fo = reinterpret_cast<float2 *>(o.fout + pol * o.fout_pol_stride + c * kNC);
            double s1 = 0.0, s2 = 0.0;
            auto epi = [&](int jj, const float2 *u) {
#pragma unroll
                for (int r = 0; r < 16; ++r) {
                    fo[jj + 1024 * r] = u[r];
                    if constexpr (MODE == 1) {
                        const double a = u[r].x, b = u[r].y;
                        s1 += a + b;
                        s2 += a * a + b * b;
                    }
                }
            };
            ifft16384(sm, TA, zin, epi);
            if constexpr (MODE == 1) {
                block_sum2(s1, s2, red);
                if (tid == 0) {
                    const double n = static_cast<double>(kNC);
                    const double mean = s1 / n;
                    double *pp = o.partials + (static_cast<int64_t>(pol) * n_chunks + c) * 3;
                    pp[0] = n;
                    pp[1] = mean;
                    pp[2] = s2 - s1 * mean;
                }
            }
        }
    }
}

// SwarmR2C alone: complex64 [n][18305] spectra (persistent over chunks).
__global__ void __launch_bounds__(kNTB, 1)
    k_swarm_r2c(const float *__restrict__ in, int64_t n_chunks, float2 *__restrict__ out, Twiddles tw) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    float2 *sm = reinterpret_cast<float2 *>(smem_raw);
    float2 *tb = sm + kPadB;
    TabsB TB = tabs_b_at(tb, tw);
    load_tabs_b(TB, tw);
    for (int64_t c = blockIdx.x; c < n_chunks; c += gridDim.x) {
        __syncthreads();
        fft18304_from_global<false>(sm, reinterpret_cast<const float2 *>(in + c * kNB), TB);
        float2 *dst = out + c * (kMB + 1);
        for (int q = threadIdx.x; q <= kMB; q += kNTB) dst[q] = r2c_bin(sm, q, __ldg(tw.w36608 + q));
    }
}

// R2dbeC2R alone: complex64 [n][18305] from bin skip -> float [n][32768].
__global__ void __launch_bounds__(kNTB, 1)
    k_r2dbe_c2r(const float2 *__restrict__ in, int64_t in_stride, int64_t n_chunks, int skip, float *__restrict__ out,
                Twiddles tw) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    float2 *sm = reinterpret_cast<float2 *>(smem_raw);
    float2 *tb = sm + kPadB;
    TabsA TA = tabs_a_at(tb);
    load_tabs_a(TA, tw);
    const int tid = threadIdx.x;
    const float2 wc = conjf2(__ldg(tw.w32768 + tid));
    for (int64_t c = blockIdx.x; c < n_chunks; c += gridDim.x) {
        __syncthreads();
        const float2 *y = in + c * in_stride + skip;
        auto zin = [&](float2 *v) {
            for_r(std::make_integer_sequence<int, 32>{}, [&](auto rc) {
                constexpr int r = decltype(rc)::value;
                const int k = tid + 512 * r;
                v[r] = c2r_pre(__ldg(y + k), __ldg(y + kMA - k), k, c2r_tw<r>(wc));
            });
        };
        float2 *dst = reinterpret_cast<float2 *>(out + c * kNC);
        auto epi = [&](int jj, const float2 *u) {
#pragma unroll
            for (int r = 0; r < 16; ++r) dst[jj + 1024 * r] = u[r];
        };
        ifft16384(sm, TA, zin, epi);
    }
}

// ---------------------------------------------------------------------------
// Threshold from the per-chunk partials: Chan's merge in FP64, in chunk order
// (deterministic).  thr_state: [0..1] effective threshold, [2..3] effective
// offset, [4..5] own threshold, [6..7] own offset.
struct Moments {
    double n, mean, m2;
};

// Chan et al. pairwise merge of (n, mean, M2).
__device__ __forceinline__ Moments merge_moments(Moments a, Moments b) {
    const double n = a.n + b.n;
    if (n == 0.0) return a;
    const double delta = b.mean - a.mean;
    return Moments{n, a.mean + delta * b.n / n, a.m2 + b.m2 + delta * delta * a.n * b.n / n};
}

// Threshold from the per-chunk partials, FP64, one warp per pol: each lane
// merges its chunks in order, then a fixed butterfly tree merges the lanes
// (deterministic).  thr_state: [0..1] effective threshold, [2..3] effective
// offset, [4..5] own threshold, [6..7] own offset.
__global__ void k_finalize_thresholds(const double *__restrict__ partials, int n_chunks, int pol1_uses_pol0,
                                      float *__restrict__ thr_state) {
    __shared__ float th_s[2], off_s[2];
    const int pol = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (pol < 2) {
        Moments m{0.0, 0.0, 0.0};
        for (int c = lane; c < n_chunks; c += 32) {
            const double *pp = partials + (static_cast<int64_t>(pol) * n_chunks + c) * 3;
            m = merge_moments(m, Moments{pp[0], pp[1], pp[2]});
        }
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            Moments other{__shfl_xor_sync(0xffffffffu, m.n, o), __shfl_xor_sync(0xffffffffu, m.mean, o),
                          __shfl_xor_sync(0xffffffffu, m.m2, o)};
            m = (lane & o) ? merge_moments(other, m) : merge_moments(m, other);
        }
        if (lane == 0) {
            th_s[pol] = static_cast<float>(sqrt(m.m2 / (m.n - 1.0)));
            off_s[pol] = static_cast<float>(m.mean);
        }
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        thr_state[4] = th_s[0];
        thr_state[5] = th_s[1];
        thr_state[6] = off_s[0];
        thr_state[7] = off_s[1];
        thr_state[0] = th_s[0];
        thr_state[1] = pol1_uses_pol0 ? th_s[0] : th_s[1];
        thr_state[2] = off_s[0];
        thr_state[3] = pol1_uses_pol0 ? off_s[0] : off_s[1];
    }
}

// Windowed thresholds: one CTA per handle, warps 0-3 pol 0 and 4-7 pol 1.
// Pushes the (n, sum, sum of squares) of each of the nb batches just
// quantized (128 chunk partials each, [pol][nb*128][3]; the first batch's
// partials are (n, mean, M2) and are converted) into the handle's FP64 ring
// (slot t mod W), then, if `update`, sets the thresholds from the sums over
// batches [max(0, T-W), T), T = t0 + nb.  Plain FP64 sums in a fixed order:
// no division but the final mean and variance.
__device__ __forceinline__ double warp_sum_d(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

__global__ void __launch_bounds__(256) k_window_update(const __grid_constant__ WinUpds U) {
    const WinUpd &u = U.u[blockIdx.x];
    __shared__ float th_s[2], off_s[2];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int pol = warp >> 2, wq = warp & 3;
    const int64_t n_chunks = static_cast<int64_t>(u.nb) * kChunks;
    for (int b = wq; b < u.nb; b += 4) {
        double n = 0.0, s1 = 0.0, s2 = 0.0;
        for (int c = lane; c < kChunks; c += 32) {
            const double *pp = u.partials + (pol * n_chunks + static_cast<int64_t>(b) * kChunks + c) * 3;
            if (u.moments) {  // (n, mean, M2)
                const double cn = pp[0], cm = pp[1];
                n += cn;
                s1 += cn * cm;
                s2 += pp[2] + cn * cm * cm;
            } else {
                n += pp[0];
                s1 += pp[1];
                s2 += pp[2];
            }
        }
        n = warp_sum_d(n);
        s1 = warp_sum_d(s1);
        s2 = warp_sum_d(s2);
        if (lane == 0) {
            double *slot = u.ring + (static_cast<int64_t>(pol) * u.W + (u.t0 + b) % u.W) * 3;
            slot[0] = n;
            slot[1] = s1;
            slot[2] = s2;
        }
    }
    __syncthreads();
    if (!u.update) return;  // uniform over the CTA
    if (wq == 0) {
        const int64_t T = u.t0 + u.nb, lo = T - u.W > 0 ? T - u.W : 0;
        double n = 0.0, s1 = 0.0, s2 = 0.0;
        for (int64_t t = lo + lane; t < T; t += 32) {
            const double *slot = u.ring + (static_cast<int64_t>(pol) * u.W + t % u.W) * 3;
            n += slot[0];
            s1 += slot[1];
            s2 += slot[2];
        }
        n = warp_sum_d(n);
        s1 = warp_sum_d(s1);
        s2 = warp_sum_d(s2);
        if (lane == 0) {
            const double mean = s1 / n;
            th_s[pol] = static_cast<float>(sqrt((s2 - s1 * mean) / (n - 1.0)));
            off_s[pol] = static_cast<float>(mean);
        }
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        float *t = u.thr;
        t[4] = th_s[0];
        t[5] = th_s[1];
        t[6] = off_s[0];
        t[7] = off_s[1];
        t[0] = th_s[0];
        t[1] = u.pol1 ? th_s[0] : th_s[1];
        t[2] = off_s[0];
        t[3] = u.pol1 ? off_s[0] : off_s[1];
    }
}

// quantize2bit over float chunks: each thread packs 16 samples into one word.
// grid (n_chunks*2048/256, 2 pols).
__global__ void k_quantize_chunks(const float *__restrict__ fin, int64_t fin_pol_stride, int64_t n_words,
                                  const float *__restrict__ thr, uint8_t *__restrict__ out, int64_t out_pol_stride,
                                  int64_t pkt_stride, int64_t payload_off, int64_t pkt0) {
    const int64_t w = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (w >= n_words) return;
    const int pol = blockIdx.y;
    const float th = thr[pol], off = thr[2 + pol];
    const float4 *src = reinterpret_cast<const float4 *>(fin + pol * fin_pol_stride + w * 16);
    uint32_t word = 0;
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        const float4 v = __ldcs(src + i);
        word |= code2(v.x, th, off) << (8 * i);
        word |= code2(v.y, th, off) << (8 * i + 2);
        word |= code2(v.z, th, off) << (8 * i + 4);
        word |= code2(v.w, th, off) << (8 * i + 6);
    }
    const int64_t c = w / kOutWords, k = w % kOutWords;
    uint32_t *dst = reinterpret_cast<uint32_t *>(out + pol * out_pol_stride + (pkt0 + c) * pkt_stride + payload_off);
    dst[k] = word;
}

// Reference-signature quantize2bit: contiguous in/out, scalar threshold.
__global__ void k_quantize_flat(const float *__restrict__ in, uint32_t *__restrict__ out, int64_t n_words, float th,
                                float off) {
    const int64_t w = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (w >= n_words) return;
    const float4 *src = reinterpret_cast<const float4 *>(in + w * 16);
    uint32_t word = 0;
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        const float4 v = __ldg(src + i);
        word |= code2(v.x, th, off) << (8 * i);
        word |= code2(v.y, th, off) << (8 * i + 2);
        word |= code2(v.z, th, off) << (8 * i + 4);
        word |= code2(v.w, th, off) << (8 * i + 6);
    }
    out[w] = word;
}

// Per-block FP64 sums for summary statistics over n floats, of the samples
// shifted by the first one (x - in[0]): a large common offset then cancels
// before the sums, not in the variance (the shifted-data algorithm; the
// finalizers add in[0] back to the mean).
__global__ void __launch_bounds__(256) k_stats_partial(const float *__restrict__ in, int64_t n,
                                                       double *__restrict__ partials) {
    __shared__ double red[64];
    const double c = __ldg(in);
    double s1 = 0.0, s2 = 0.0;
    for (int64_t i = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; i < n;
         i += static_cast<int64_t>(gridDim.x) * blockDim.x) {
        const double v = static_cast<double>(__ldg(in + i)) - c;
        s1 += v;
        s2 += v * v;
    }
    block_sum2(s1, s2, red);
    if (threadIdx.x == 0) {
        partials[2 * blockIdx.x] = s1;
        partials[2 * blockIdx.x + 1] = s2;
    }
}

// ---------------------------------------------------------------------------
// Twiddle tables, FP64 on the host then rounded to FP32.
cudaError_t build_twiddles(Twiddles &tw, float2 **storage) {
    const int sizes[4] = {kMA, kMB, kMA, kMB + 1};
    const double periods[4] = {double(kMA), double(kMB), double(kNA), double(kNB)};
    size_t total = 0;
    for (int i = 0; i < 4; ++i) total += sizes[i];
    std::vector<float2> host(total);
    size_t off = 0;
    size_t offs[4];
    for (int t = 0; t < 4; ++t) {
        offs[t] = off;
        for (int k = 0; k < sizes[t]; ++k) {
            const double a = -2.0 * M_PI * static_cast<double>(k) / periods[t];
            host[off + k] = make_float2(static_cast<float>(std::cos(a)), static_cast<float>(std::sin(a)));
        }
        off += sizes[t];
    }
    float2 *d = nullptr;
    cudaError_t e = cudaMalloc(&d, total * sizeof(float2));
    if (e != cudaSuccess) return e;
    e = cudaMemcpy(d, host.data(), total * sizeof(float2), cudaMemcpyHostToDevice);
    if (e != cudaSuccess) {
        cudaFree(d);
        return e;
    }
    tw.w16384 = d + offs[0];
    tw.w18304 = d + offs[1];
    tw.w32768 = d + offs[2];
    tw.w36608 = d + offs[3];
    *storage = d;
    return cudaSuccess;
}

cudaError_t configure_fft_kernels() {
    cudaError_t e;
    if ((e = cudaFuncSetAttribute(k_swarm_c2r, cudaFuncAttributeMaxDynamicSharedMemorySize, int(kSmemA))) != cudaSuccess)
        return e;
    if ((e = cudaFuncSetAttribute(k_resample<0>, cudaFuncAttributeMaxDynamicSharedMemorySize, int(kSmemB))) != cudaSuccess)
        return e;
    if ((e = cudaFuncSetAttribute(k_resample<3>, cudaFuncAttributeMaxDynamicSharedMemorySize, int(kSmemB))) != cudaSuccess)
        return e;
    if ((e = cudaFuncSetAttribute(k_resample<1>, cudaFuncAttributeMaxDynamicSharedMemorySize, int(kSmemB))) != cudaSuccess)
        return e;
    if ((e = cudaFuncSetAttribute(k_resample<2>, cudaFuncAttributeMaxDynamicSharedMemorySize, int(kSmemB))) != cudaSuccess)
        return e;
    if ((e = cudaFuncSetAttribute(k_swarm_r2c, cudaFuncAttributeMaxDynamicSharedMemorySize, int(kSmemB))) != cudaSuccess)
        return e;
    if ((e = cudaFuncSetAttribute(k_r2dbe_c2r, cudaFuncAttributeMaxDynamicSharedMemorySize, int(kSmemB))) != cudaSuccess)
        return e;
    return cudaSuccess;
}

// Persistent grid size: one CTA per SM, at most `items`.
static unsigned persistent_grid(int64_t items) {
    int dev = 0, sms = 0;
    if (cudaGetDevice(&dev) != cudaSuccess ||
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || sms <= 0) {
        cudaGetLastError();
        sms = 1;
    }
    return static_cast<unsigned>(items < sms ? items : sms);
}

// ---- launchers ----------------------------------------------------------------
cudaError_t launch_swarm_c2r_segs(const SegsA &S, const Twiddles &tw, cudaStream_t st) {
    if (S.n_items <= 0) return cudaSuccess;
    if (S.n < 1 || S.n > kMaxSegs) return cudaErrorInvalidValue;
    k_swarm_c2r<<<persistent_grid(S.n_items), kNTA, kSmemA, st>>>(S, tw);
    return cudaGetLastError();
}

cudaError_t launch_resample_segs(int mode, const SegsB &S, const Twiddles &tw, cudaStream_t st) {
    if (S.n_items <= 0) return cudaSuccess;
    if (S.n < 1 || S.n > kMaxSegs) return cudaErrorInvalidValue;
    const unsigned grid = persistent_grid(S.n_items);
    if (mode == 0)
        k_resample<0><<<grid, kNTB, kSmemB, st>>>(S, tw);
    else if (mode == 3)
        k_resample<3><<<grid, kNTB, kSmemB, st>>>(S, tw);
    else if (mode == 1)
        k_resample<1><<<grid, kNTB, kSmemB, st>>>(S, tw);
    else
        k_resample<2><<<grid, kNTB, kSmemB, st>>>(S, tw);
    return cudaGetLastError();
}

cudaError_t launch_swarm_c2r(const uint32_t *spec, int64_t spec_pol_stride, int64_t snap0, int64_t n_snaps, int n_pols,
                             float *out, int64_t out_pol_stride, const Twiddles &tw, cudaStream_t st) {
    if (n_snaps <= 0) return cudaSuccess;
    SegsA S{};
    S.n = 1;
    S.n_items = n_snaps * n_pols;
    S.s[0] = SegA{spec, out, spec_pol_stride, snap0, n_snaps, out_pol_stride, 0};
    return launch_swarm_c2r_segs(S, tw, st);
}

cudaError_t launch_resample(int mode, const float *in, int64_t in_pol_stride, int skip, int64_t n_chunks, int n_pols,
                            const ResampleOut &o, const Twiddles &tw, cudaStream_t st) {
    if (n_chunks <= 0) return cudaSuccess;
    SegsB S{};
    S.n = 1;
    S.n_items = n_chunks * n_pols;
    S.s[0] = SegB{in, in_pol_stride, 0, static_cast<int>(n_chunks), skip, o};
    return launch_resample_segs(mode, S, tw, st);
}

cudaError_t launch_swarm_r2c(const float *in, int64_t n_chunks, void *out, const Twiddles &tw, cudaStream_t st) {
    if (n_chunks <= 0) return cudaSuccess;
    k_swarm_r2c<<<persistent_grid(n_chunks), kNTB, kSmemB, st>>>(in, n_chunks, static_cast<float2 *>(out), tw);
    return cudaGetLastError();
}

cudaError_t launch_r2dbe_c2r(const void *in, int64_t in_stride, int64_t n_chunks, int skip, float *out,
                             const Twiddles &tw, cudaStream_t st) {
    if (n_chunks <= 0) return cudaSuccess;
    k_r2dbe_c2r<<<persistent_grid(n_chunks), kNTB, kSmemB, st>>>(static_cast<const float2 *>(in), in_stride, n_chunks,
                                                                  skip, out, tw);
    return cudaGetLastError();
}

cudaError_t launch_window_update(const WinUpds &U, cudaStream_t st) {
    if (U.n <= 0) return cudaSuccess;
    if (U.n > kMaxSegs) return cudaErrorInvalidValue;
    k_window_update<<<U.n, 256, 0, st>>>(U);
    return cudaGetLastError();
}

cudaError_t launch_finalize_thresholds(const double *partials, int n_chunks, int pol1_uses_pol0, float *thr_state,
                                       cudaStream_t st) {
    k_finalize_thresholds<<<1, 64, 0, st>>>(partials, n_chunks, pol1_uses_pol0, thr_state);
    return cudaGetLastError();
}

cudaError_t launch_quantize_chunks(const float *fin, int64_t fin_pol_stride, int64_t n_chunks, const float *thr,
                                   uint8_t *out, int64_t out_pol_stride, int64_t pkt_stride, int64_t payload_off,
                                   int64_t pkt0, cudaStream_t st) {
    const int64_t n_words = n_chunks * kOutWords;
    if (n_words <= 0) return cudaSuccess;
    dim3 grid(static_cast<unsigned>((n_words + 255) / 256), 2);
    k_quantize_chunks<<<grid, 256, 0, st>>>(fin, fin_pol_stride, n_words, thr, out, out_pol_stride, pkt_stride,
                                            payload_off, pkt0);
    return cudaGetLastError();
}

cudaError_t launch_quantize_flat(const float *in, uint32_t *out, int64_t n, float th, float off, cudaStream_t st) {
    const int64_t n_words = n / 16;
    if (n_words <= 0) return cudaSuccess;
    k_quantize_flat<<<static_cast<unsigned>((n_words + 255) / 256), 256, 0, st>>>(in, out, n_words, th, off);
    return cudaGetLastError();
}

int stats_partial_blocks(int64_t n) {
    int64_t b = (n + 255) / 256;
    return static_cast<int>(b < 1216 ? (b < 1 ? 1 : b) : 1216);
}

cudaError_t launch_stats_partial(const float *in, int64_t n, double *partials, int blocks, cudaStream_t st) {
    k_stats_partial<<<blocks, 256, 0, st>>>(in, n, partials);
    return cudaGetLastError();
}

}  // namespace sdbe
