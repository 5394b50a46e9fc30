// Resampling FFT kernels, one CTA per transform, data resident in shared memory.
//
// Reference: the three cuFFT plans of vdif_inout_gpu_thread.cu:271-333 run by
// SwarmC2R / SwarmR2C / R2dbeC2R (:589-709) on each 143-snapshot batch.
//   stage A  C2R 32768 per snapshot  = 16384-point complex inverse FFT plus
//            Hermitian pre-processing, fed straight from the packed 2-bit
//            spectrum (beng_int8_to_cufftComplex and the Nyquist memset fused).
//   stage BC R2C 36608 per chunk = 18304-point complex FFT + post-processing,
//            bins [skip, skip+16384] selected in registers, C2R 32768 through
//            a 16384-point inverse FFT, then quantize2bit in the epilogue.
// All scaling is cuFFT's unnormalised convention.
#include <vector>
#include <cmath>

#include "fft_core.cuh"
#include "launchers.cuh"
#include "sdbe_internal.cuh"

namespace sdbe {

constexpr int kNTA = 512;   // stage A threads: 512 radix-32 butterflies per pass
constexpr int kNTB = 576;   // stage BC threads: balances the 16/8/11/13 passes of 18304
constexpr int kPadA = padded_len(kMA);
constexpr int kPadB = padded_len(kMB);
constexpr size_t kSmemA = kGroups * sizeof(uint32_t) + kPadA * sizeof(float2);
constexpr size_t kSmemB = kPadB * sizeof(float2);

// ---------------------------------------------------------------------------
// Inverse 16384-point FFT, radices 32 x 32 x 16 (Stockham).  zin(k) gives input
// k (it may read `sm`; the first barrier separates those reads from the
// writes), epi(jj, u) receives outputs z[jj + 1024 r], r < 16.  blockDim.x is
// a multiple of 32 and >= 512.
template <class In, class Epi>
__device__ __forceinline__ void ifft16384(float2 *sm, const float2 *__restrict__ w16384, In zin, Epi epi) {
    const int tid = threadIdx.x;
    float2 v[32];
    if (tid < 512) {
#pragma unroll
        for (int r = 0; r < 32; ++r) v[r] = zin(tid + 512 * r);
        dft<32, true>(v);
    }
    __syncthreads();
    if (tid < 512) {
#pragma unroll
        for (int r = 0; r < 32; ++r) sm[pad(32 * tid + r)] = v[r];
    }
    __syncthreads();
    if (tid < 512) {
#pragma unroll
        for (int r = 0; r < 32; ++r) v[r] = sm[pad(tid + 512 * r)];
        const int jm = tid & 31;
#pragma unroll
        for (int r = 1; r < 32; ++r) v[r] = cmul(v[r], twiddle<true>(w16384, jm * r * 16));
        dft<32, true>(v);
    }
    __syncthreads();
    if (tid < 512) {
        const int base = (tid >> 5) * 1024 + (tid & 31);
#pragma unroll
        for (int r = 0; r < 32; ++r) sm[pad(base + 32 * r)] = v[r];
    }
    __syncthreads();
    for (int jj = tid; jj < 1024; jj += blockDim.x) {
        float2 u[16];
#pragma unroll
        for (int r = 0; r < 16; ++r) u[r] = sm[pad(jj + 1024 * r)];
#pragma unroll
        for (int r = 1; r < 16; ++r) u[r] = cmul(u[r], twiddle<true>(w16384, jj * r));
        dft<16, true>(u);
        epi(jj, u);
    }
}

// In-place Stockham pass in shared memory: every thread first holds all of
// its butterflies in registers, then all threads write after a barrier.
template <int R, int NS, int N, int NT, bool INV>
__device__ __forceinline__ void smem_pass(float2 *sm, const float2 *__restrict__ tw) {
    constexpr int NB = N / R;
    constexpr int ITERS = (NB + NT - 1) / NT;
    constexpr int TS = N / (NS * R);
    float2 v[ITERS][R];
#pragma unroll
    for (int it = 0; it < ITERS; ++it) {
        const int j = threadIdx.x + it * NT;
        if (j < NB) {
#pragma unroll
            for (int r = 0; r < R; ++r) v[it][r] = sm[pad(j + NB * r)];
            const int jm = j % NS;
#pragma unroll
            for (int r = 1; r < R; ++r) v[it][r] = cmul(v[it][r], twiddle<INV>(tw, jm * r * TS));
            dft<R, INV>(v[it]);
        }
    }
    __syncthreads();
#pragma unroll
    for (int it = 0; it < ITERS; ++it) {
        const int j = threadIdx.x + it * NT;
        if (j < NB) {
            const int base = (j / NS) * NS * R + (j % NS);
#pragma unroll
            for (int r = 0; r < R; ++r) sm[pad(base + NS * r)] = v[it][r];
        }
    }
    __syncthreads();
}

// Forward 18304-point FFT of the complex sequence z[m] = x[2m] + i x[2m+1]
// read from global memory; result Z in natural order in `sm`.
// Radices 16 (from global) x 8 x 11 x 13.
__device__ __forceinline__ void fft18304_from_global(float2 *sm, const float2 *__restrict__ z,
                                                     const float2 *__restrict__ w18304) {
    constexpr int NB1 = kMB / 16;  // 1144
    for (int j = threadIdx.x; j < NB1; j += kNTB) {
        float2 v[16];
#pragma unroll
        for (int r = 0; r < 16; ++r) v[r] = __ldcs(z + j + NB1 * r);
        dft<16, false>(v);
#pragma unroll
        for (int r = 0; r < 16; ++r) sm[pad(16 * j + r)] = v[r];
    }
    __syncthreads();
    smem_pass<8, 16, kMB, kNTB, false>(sm, w18304);
    smem_pass<11, 128, kMB, kNTB, false>(sm, w18304);
    smem_pass<13, 1408, kMB, kNTB, false>(sm, w18304);
}

// Unnormalised R2C bin q (0 <= q <= 18304) of the 36608 real samples from the
// half-length complex transform Z in `sm`:
//   X[q] = (Z[q] + conj Z[M-q])/2 - i W^q (Z[q] - conj Z[M-q])/2,  W = e^{-2 pi i/36608}.
__device__ __forceinline__ float2 r2c_bin(const float2 *sm, const float2 *__restrict__ w36608, int q) {
    const int qa = q == kMB ? 0 : q;
    const int qb = q == 0 ? 0 : kMB - q;
    const float2 za = sm[pad(qa)];
    const float2 zb = conjf2(sm[pad(qb)]);
    const float2 s = cadd(za, zb), d = csub(za, zb);
    const float2 wd = cmul(__ldg(w36608 + q), d);
    return make_float2(0.5f * (s.x + wd.y), 0.5f * (s.y - wd.x));
}

// Hermitian pre-processing of a C2R of length 32768 from bins Y[0..16384]:
//   Z[k] = (Y[k] + conj Y[M-k]) + i e^{+2 pi i k/32768} (Y[k] - conj Y[M-k]),
// imaginary parts of Y[0] and Y[16384] ignored (as cuFFT / numpy do).
__device__ __forceinline__ float2 c2r_pre(float2 y, float2 ym, int k, const float2 *__restrict__ w32768) {
    if (k == 0) {
        y.y = 0.f;
        ym.y = 0.f;
    }
    const float2 e = make_float2(y.x + ym.x, y.y - ym.y);
    const float2 o = cmul(make_float2(y.x - ym.x, y.y + ym.y), twiddle<true>(w32768, k));
    return make_float2(e.x - o.y, e.y + o.x);
}

// Packed nibble -> (real, imag) = codes - 2.
__device__ __forceinline__ float2 nib_value(const uint32_t *sp, int k) {
    const uint32_t nib = (sp[k >> 3] >> ((k & 7) * 4)) & 0xFu;
    return make_float2(static_cast<float>(nib >> 2) - 2.0f, static_cast<float>(nib & 3u) - 2.0f);
}

// ---------------------------------------------------------------------------
// Stage A: grid (n_snaps, 2 pols).  Packed spectrum of snapshot s of pol p at
// spec + p*spec_pol_stride + (snap0 + s)*2048; time series to
// out + p*out_pol_stride + s*32768.
__global__ void __launch_bounds__(kNTA, 1)
    k_swarm_c2r(const uint32_t *__restrict__ spec, int64_t spec_pol_stride, int64_t snap0,
                float *__restrict__ out, int64_t out_pol_stride, Twiddles tw) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    uint32_t *sp = reinterpret_cast<uint32_t *>(smem_raw);
    float2 *sm = reinterpret_cast<float2 *>(smem_raw + kGroups * sizeof(uint32_t));
    const int pol = blockIdx.y;
    const int64_t s = blockIdx.x;
    const uint4 *src = reinterpret_cast<const uint4 *>(spec + pol * spec_pol_stride + (snap0 + s) * kGroups);
    reinterpret_cast<uint4 *>(sp)[threadIdx.x] = __ldg(src + threadIdx.x);  // 512 x 16 B = 8 KB
    __syncthreads();
    float2 *dst = reinterpret_cast<float2 *>(out + pol * out_pol_stride + s * kNA);
    const float2 *w32768 = tw.w32768;
    auto zin = [&](int k) -> float2 {
        const float2 a = nib_value(sp, k);
        const float2 b = k == 0 ? make_float2(0.f, 0.f) : nib_value(sp, kMA - k);  // X[16384] = 0
        return c2r_pre(a, b, k, w32768);
    };
    auto epi = [&](int jj, const float2 *u) {
#pragma unroll
        for (int r = 0; r < 16; ++r) dst[jj + 1024 * r] = u[r];
    };
    ifft16384(sm, tw.w16384, zin, epi);
}

// ---------------------------------------------------------------------------
// Stage BC: grid (n_chunks, 2 pols).  Chunk c of pol p: 36608 floats at
// in + p*in_pol_stride + c*36608.
//   MODE 0: quantize with thr[p] / thr[2+p] into the u32 payload at
//           out + p*out_pol_stride + (pkt0 + c)*pkt_stride + payload_off.
//   MODE 1: floats to fout + p*fout_pol_stride + c*32768 and per-chunk
//           (n, mean, M2) in FP64 to partials[(p*n_chunks + c)*3].
//   MODE 2: floats only.

template <int MODE>
__global__ void __launch_bounds__(kNTB, 1)
    k_resample(const float *__restrict__ in, int64_t in_pol_stride, int skip, int n_chunks, ResampleOut o,
               Twiddles tw) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    float2 *sm = reinterpret_cast<float2 *>(smem_raw);
    __shared__ double red[64];
    const int pol = blockIdx.y;
    const int64_t c = blockIdx.x;
    const float2 *z = reinterpret_cast<const float2 *>(in + pol * in_pol_stride + c * kNB);
    fft18304_from_global(sm, z, tw.w18304);

    const float2 *w36608 = tw.w36608, *w32768 = tw.w32768;
    auto zin = [&](int jj) -> float2 {
        const float2 y = r2c_bin(sm, w36608, skip + jj);
        const float2 ym = r2c_bin(sm, w36608, skip + kMA - jj);
        return c2r_pre(y, ym, jj, w32768);
    };
    if constexpr (MODE == 0) {
        uint32_t *words = reinterpret_cast<uint32_t *>(o.out + pol * o.out_pol_stride + (o.pkt0 + c) * o.pkt_stride +
                                                       o.payload_off);
        const float th = o.thr[pol], off = o.thr[2 + pol];
        auto epi = [&](int jj, const float2 *u) {
#pragma unroll
            for (int r = 0; r < 16; ++r) {
                uint32_t q = (code2(u[r].x, th, off) | (code2(u[r].y, th, off) << 2)) << (4 * (jj & 7));
                q |= __shfl_xor_sync(0xffffffffu, q, 1);
                q |= __shfl_xor_sync(0xffffffffu, q, 2);
                q |= __shfl_xor_sync(0xffffffffu, q, 4);
                if ((jj & 7) == 0) words[(jj >> 3) + 128 * r] = q;
            }
        };
        ifft16384(sm, tw.w16384, zin, epi);
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
        ifft16384(sm, tw.w16384, zin, epi);
        if constexpr (MODE == 1) {
            block_sum2(s1, s2, red);
            if (threadIdx.x == 0) {
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

// SwarmR2C alone: complex64 [n][18305] spectra.  grid (n_chunks).
__global__ void __launch_bounds__(kNTB, 1)
    k_swarm_r2c(const float *__restrict__ in, float2 *__restrict__ out, Twiddles tw) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    float2 *sm = reinterpret_cast<float2 *>(smem_raw);
    const int64_t c = blockIdx.x;
    fft18304_from_global(sm, reinterpret_cast<const float2 *>(in + c * kNB), tw.w18304);
    float2 *dst = out + c * (kMB + 1);
    for (int q = threadIdx.x; q <= kMB; q += kNTB) dst[q] = r2c_bin(sm, tw.w36608, q);
}

// R2dbeC2R alone: complex64 [n][18305] from bin skip -> float [n][32768].
__global__ void __launch_bounds__(kNTB, 1)
    k_r2dbe_c2r(const float2 *__restrict__ in, int skip, float *__restrict__ out, Twiddles tw) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    float2 *sm = reinterpret_cast<float2 *>(smem_raw);
    const int64_t c = blockIdx.x;
    const float2 *y = in + c * (kMB + 1) + skip;
    const float2 *w32768 = tw.w32768;
    auto zin = [&](int k) -> float2 { return c2r_pre(__ldg(y + k), __ldg(y + kMA - k), k, w32768); };
    float2 *dst = reinterpret_cast<float2 *>(out + c * kNC);
    auto epi = [&](int jj, const float2 *u) {
#pragma unroll
        for (int r = 0; r < 16; ++r) dst[jj + 1024 * r] = u[r];
    };
    ifft16384(sm, tw.w16384, zin, epi);
}

// ---------------------------------------------------------------------------
// Threshold from the per-chunk partials: Chan's merge in FP64, in chunk order
// (deterministic).  thr_state: [0..1] effective threshold, [2..3] effective
// offset, [4..5] own threshold, [6..7] own offset.
__global__ void k_finalize_thresholds(const double *__restrict__ partials, int n_chunks, int pol1_uses_pol0,
                                      float *__restrict__ thr_state) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    float th[2], off[2];
    for (int pol = 0; pol < 2; ++pol) {
        double n = 0.0, mean = 0.0, m2 = 0.0;
        for (int c = 0; c < n_chunks; ++c) {
            const double *pp = partials + (static_cast<int64_t>(pol) * n_chunks + c) * 3;
            const double nb = pp[0], mb = pp[1], m2b = pp[2];
            const double nn = n + nb;
            const double delta = mb - mean;
            mean += delta * nb / nn;
            m2 += m2b + delta * delta * n * nb / nn;
            n = nn;
        }
        th[pol] = static_cast<float>(sqrt(m2 / (n - 1.0)));
        off[pol] = static_cast<float>(mean);
    }
    thr_state[4] = th[0];
    thr_state[5] = th[1];
    thr_state[6] = off[0];
    thr_state[7] = off[1];
    thr_state[0] = th[0];
    thr_state[1] = pol1_uses_pol0 ? th[0] : th[1];
    thr_state[2] = off[0];
    thr_state[3] = pol1_uses_pol0 ? off[0] : off[1];
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

// Per-block FP64 sums for summary statistics over n floats.
__global__ void __launch_bounds__(256) k_stats_partial(const float *__restrict__ in, int64_t n,
                                                       double *__restrict__ partials) {
    __shared__ double red[64];
    double s1 = 0.0, s2 = 0.0;
    for (int64_t i = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; i < n;
         i += static_cast<int64_t>(gridDim.x) * blockDim.x) {
        const double v = __ldg(in + i);
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

// ---- launchers ----------------------------------------------------------------
cudaError_t launch_swarm_c2r(const uint32_t *spec, int64_t spec_pol_stride, int64_t snap0, int64_t n_snaps, int n_pols,
                             float *out, int64_t out_pol_stride, const Twiddles &tw, cudaStream_t st) {
    if (n_snaps <= 0) return cudaSuccess;
    dim3 grid(static_cast<unsigned>(n_snaps), n_pols);
    k_swarm_c2r<<<grid, kNTA, kSmemA, st>>>(spec, spec_pol_stride, snap0, out, out_pol_stride, tw);
    return cudaGetLastError();
}

cudaError_t launch_resample(int mode, const float *in, int64_t in_pol_stride, int skip, int64_t n_chunks, int n_pols,
                            const ResampleOut &o, const Twiddles &tw, cudaStream_t st) {
    if (n_chunks <= 0) return cudaSuccess;
    dim3 grid(static_cast<unsigned>(n_chunks), n_pols);
    const int nc = static_cast<int>(n_chunks);
    if (mode == 0)
        k_resample<0><<<grid, kNTB, kSmemB, st>>>(in, in_pol_stride, skip, nc, o, tw);
    else if (mode == 1)
        k_resample<1><<<grid, kNTB, kSmemB, st>>>(in, in_pol_stride, skip, nc, o, tw);
    else
        k_resample<2><<<grid, kNTB, kSmemB, st>>>(in, in_pol_stride, skip, nc, o, tw);
    return cudaGetLastError();
}

cudaError_t launch_swarm_r2c(const float *in, int64_t n_chunks, void *out, const Twiddles &tw, cudaStream_t st) {
    if (n_chunks <= 0) return cudaSuccess;
    k_swarm_r2c<<<static_cast<unsigned>(n_chunks), kNTB, kSmemB, st>>>(in, static_cast<float2 *>(out), tw);
    return cudaGetLastError();
}

cudaError_t launch_r2dbe_c2r(const void *in, int64_t n_chunks, int skip, float *out, const Twiddles &tw,
                             cudaStream_t st) {
    if (n_chunks <= 0) return cudaSuccess;
    k_r2dbe_c2r<<<static_cast<unsigned>(n_chunks), kNTB, kSmemB, st>>>(static_cast<const float2 *>(in), skip, out,
                                                                        tw);
    return cudaGetLastError();
}

cudaError_t launch_finalize_thresholds(const double *partials, int n_chunks, int pol1_uses_pol0, float *thr_state,
                                       cudaStream_t st) {
    k_finalize_thresholds<<<1, 32, 0, st>>>(partials, n_chunks, pol1_uses_pol0, thr_state);
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
