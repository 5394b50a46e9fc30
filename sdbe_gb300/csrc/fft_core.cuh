// Register-resident DFT codelets and shared-memory helpers for the
// Stockham FFT passes of the resampling kernels.
//
// A pass of radix R over an N-point sequence held in shared memory
// (Stockham autosort, natural order in and out):
//   for butterfly j < N/R:  v[r] = x[j + r*N/R]
//                           v[r] *= W_{Ns*R}^{(j mod Ns)*r}
//                           v = DFT_R(v)
//                           y[(j/Ns)*Ns*R + (j mod Ns) + r*Ns] = v[r]
// with Ns the product of the radices of the earlier passes.  The first pass
// therefore reads with stride N/R (coalesced straight from global memory)
// and the last pass writes with stride N/R (coalesced straight to global).
#pragma once

#include "sdbe_internal.cuh"

namespace sdbe {

// Padded shared-memory index: one float2 of padding per 32 elements keeps
// the stride-16/32 accesses of the passes free of bank conflicts.
__device__ __forceinline__ int pad(int a) { return a + (a >> 5); }
constexpr int padded_len(int n) { return n + (n >> 5) + 1; }

// cos(2 pi m / 32) for integer m; constant-folds when m is a compile-time value.
__device__ __forceinline__ float cos32(int m) {
    m &= 31;
    constexpr float t[9] = {1.0f, 0.98078528040323043f, 0.92387953251128674f,
                            0.83146961230254524f, 0.70710678118654757f, 0.55557023301960229f,
                            0.38268343236508984f, 0.19509032201612833f, 0.0f};
    if (m <= 8) return t[m];
    if (m <= 16) return -t[16 - m];
    if (m <= 24) return -t[m - 16];
    return t[32 - m];
}
__device__ __forceinline__ float sin32(int m) { return cos32(m - 8); }

// a * W_32^m, W_32 = exp(-2 pi i / 32) (forward) or its conjugate (inverse).
template <bool INV>
__device__ __forceinline__ float2 mul_w32(float2 a, int m) {
    m &= 31;
    if (m == 0) return a;
    if (m == 16) return make_float2(-a.x, -a.y);
    if (m == 8) return INV ? make_float2(-a.y, a.x) : make_float2(a.y, -a.x);
    if (m == 24) return INV ? make_float2(a.y, -a.x) : make_float2(-a.y, a.x);
    const float c = cos32(m);
    const float s = INV ? sin32(m) : -sin32(m);
    return make_float2(a.x * c - a.y * s, a.x * s + a.y * c);
}

__host__ __device__ constexpr int ilog2c(int n) { return n <= 1 ? 0 : 1 + ilog2c(n >> 1); }
__host__ __device__ constexpr int bitrev(int x, int bits) {
    int r = 0;
    for (int b = 0; b < bits; ++b) r |= ((x >> b) & 1) << (bits - 1 - b);
    return r;
}

// In-register power-of-two DFT (R <= 32), natural order in and out:
// bit-reversal by register renaming, then radix-2 decimation-in-time stages.
template <int R, bool INV>
__device__ __forceinline__ void dft_pow2(float2 *v) {
    constexpr int B = ilog2c(R);
#pragma unroll
    for (int i = 0; i < R; ++i) {
        const int j = bitrev(i, B);
        if (i < j) {
            const float2 t = v[i];
            v[i] = v[j];
            v[j] = t;
        }
    }
#pragma unroll
    for (int half = 1; half < R; half <<= 1) {
#pragma unroll
        for (int i = 0; i < R; i += 2 * half) {
#pragma unroll
            for (int k = 0; k < half; ++k) {
                const float2 b = mul_w32<INV>(v[i + k + half], k * (32 / (2 * half)));
                const float2 a = v[i + k];
                v[i + k] = cadd(a, b);
                v[i + k + half] = csub(a, b);
            }
        }
    }
}

// cos/sin(2 pi m / P) tables for the odd prime radices.
template <int P>
struct OddConst;
template <>
struct OddConst<11> {
    __device__ static __forceinline__ float c(int m) {
        constexpr float t[6] = {1.0f, 0.84125353283118121f, 0.41541501300188644f, -0.142314838273285f,
                                -0.65486073394528499f, -0.95949297361449737f};
        return t[m];
    }
    __device__ static __forceinline__ float s(int m) {
        constexpr float t[6] = {0.0f, 0.54064081745559756f, 0.90963199535451833f, 0.9898214418809328f,
                                0.75574957435425827f, 0.28173255684142967f};
        return t[m];
    }
};
template <>
struct OddConst<13> {
    __device__ static __forceinline__ float c(int m) {
        constexpr float t[7] = {1.0f, 0.88545602565320991f, 0.56806474673115592f, 0.12053668025532301f,
                                -0.35460488704253545f, -0.74851074817110119f, -0.97094181742605201f};
        return t[m];
    }
    __device__ static __forceinline__ float s(int m) {
        constexpr float t[7] = {0.0f, 0.46472317204376851f, 0.82298386589365635f, 0.99270887409805397f,
                                0.93501624268541483f, 0.66312265824079519f, 0.23931566428755768f};
        return t[m];
    }
};

// Odd prime DFT by conjugate-pair symmetry: with s_j = v_j + v_{P-j},
// d_j = v_j - v_{P-j}, A_k = v_0 + sum s_j cos(2 pi jk/P),
// B_k = sum d_j sin(2 pi jk/P):  y_k = A_k -+ i B_k, y_{P-k} = A_k +- i B_k.
template <int P, bool INV>
__device__ __forceinline__ void dft_odd(float2 *v) {
    constexpr int H = (P - 1) / 2;
    float2 s[H + 1], d[H + 1];
#pragma unroll
    for (int j = 1; j <= H; ++j) {
        s[j] = cadd(v[j], v[P - j]);
        d[j] = csub(v[j], v[P - j]);
    }
    float2 y0 = v[0];
#pragma unroll
    for (int j = 1; j <= H; ++j) y0 = cadd(y0, s[j]);
    float2 out[P];
    out[0] = y0;
#pragma unroll
    for (int k = 1; k <= H; ++k) {
        float2 A = v[0];
        float2 Bv = make_float2(0.f, 0.f);
#pragma unroll
        for (int j = 1; j <= H; ++j) {
            int m = (j * k) % P;
            float cs, sn;
            if (m <= H) {
                cs = OddConst<P>::c(m);
                sn = OddConst<P>::s(m);
            } else {
                cs = OddConst<P>::c(P - m);
                sn = -OddConst<P>::s(P - m);
            }
            A.x = fmaf(s[j].x, cs, A.x);
            A.y = fmaf(s[j].y, cs, A.y);
            Bv.x = fmaf(d[j].x, sn, Bv.x);
            Bv.y = fmaf(d[j].y, sn, Bv.y);
        }
        // forward: y_k = A - i B = (A.x + B.y, A.y - B.x)
        if (!INV) {
            out[k] = make_float2(A.x + Bv.y, A.y - Bv.x);
            out[P - k] = make_float2(A.x - Bv.y, A.y + Bv.x);
        } else {
            out[k] = make_float2(A.x - Bv.y, A.y + Bv.x);
            out[P - k] = make_float2(A.x + Bv.y, A.y - Bv.x);
        }
    }
#pragma unroll
    for (int k = 0; k < P; ++k) v[k] = out[k];
}

template <int R, bool INV>
__device__ __forceinline__ void dft(float2 *v) {
    if constexpr (R == 11 || R == 13) {
        dft_odd<R, INV>(v);
    } else {
        dft_pow2<R, INV>(v);
    }
}

// ---- compile-time twiddle constants ---------------------------------------
// sin/cos of 2*pi*num/den in double at compile time: exact integer reduction
// to a quadrant, then Taylor series on |x| <= pi/4 (error < 1e-16).
constexpr double kPi = 3.141592653589793238462643383279502884;
__host__ __device__ constexpr double cx_sin_small(double x) {
    double x2 = x * x, term = x, sum = x;
    for (int k = 1; k < 14; ++k) {
        term *= -x2 / ((2.0 * k) * (2.0 * k + 1.0));
        sum += term;
    }
    return sum;
}
__host__ __device__ constexpr double cx_cos_small(double x) {
    double x2 = x * x, term = 1.0, sum = 1.0;
    for (int k = 1; k < 14; ++k) {
        term *= -x2 / ((2.0 * k - 1.0) * (2.0 * k));
        sum += term;
    }
    return sum;
}
// Returns {cos, sin} of 2*pi*num/den.
struct CS {
    double c, s;
};
__host__ __device__ constexpr CS cx_cossin_2pi(long long num, long long den) {
    long long m = num % den;
    if (m < 0) m += den;
    // 8m/den in [0, 8): octant index q = round(4m/den) in [0, 4], remainder t in [-1/2, 1/2]
    const long long q4 = (8 * m + den) / (2 * den);       // nearest quarter-turn
    const double t = (4.0 * static_cast<double>(m) - static_cast<double>(q4) * static_cast<double>(den)) /
                     static_cast<double>(den);          // fraction of a quarter-turn
    const double x = t * (kPi / 2.0);
    const double sx = cx_sin_small(x), cxv = cx_cos_small(x);
    switch (q4 & 3) {
        case 0: return CS{cxv, sx};
        case 1: return CS{-sx, cxv};
        case 2: return CS{-cxv, -sx};
        default: return CS{sx, -cxv};
    }
}
// W_N^E = exp(-2 pi i E/N) rounded to float, usable as device constants.
template <long long N, long long E>
struct TwC {
    static constexpr CS v = cx_cossin_2pi(E, N);
    static constexpr float c = static_cast<float>(v.c);
    static constexpr float s = static_cast<float>(-v.s);
};
// a * W_N^E (or a * conj(W_N^E) when CONJ) with E a compile-time value.
template <long long N, long long E, bool CONJ>
__device__ __forceinline__ float2 mul_tc(float2 a) {
    constexpr float c = TwC<N, E>::c;
    constexpr float s = CONJ ? -TwC<N, E>::s : TwC<N, E>::s;
    if constexpr (E % N == 0) {
        return a;
    } else {
        return make_float2(a.x * c - a.y * s, a.x * s + a.y * c);
    }
}

// Padded index of the small shared-memory twiddle tables.
__device__ __forceinline__ int tp(int m) { return m + (m >> 4); }
constexpr int tp_len(int n) { return n + ((n - 1) >> 4) + 1; }

// W_N^e from the two-level tables H[a] = W_N^{128 a}, L[b] = W_N^b.
__device__ __forceinline__ float2 tw2(const float2 *H, const float2 *L, int e) {
    return cmul(H[tp(e >> 7)], L[tp(e & 127)]);
}

// Table twiddle W_N^e (forward) or its conjugate (inverse).
template <bool INV>
__device__ __forceinline__ float2 twiddle(const float2 *__restrict__ tab, int e) {
    const float2 w = __ldg(tab + e);
    return INV ? make_float2(w.x, -w.y) : w;
}

// ---- 2-bit requantization (quantize2bit, vdif_inout_gpu_thread.cu:577) ----
__device__ __forceinline__ uint32_t code2(float x, float th, float off) {
    const float v = x - off;
    return ((static_cast<uint32_t>(fabsf(v) >= th) | 2u) ^ (3u * static_cast<uint32_t>(v < 0.f))) & 3u;
}

// 8 x 8 transpose of 4-bit nibbles over the aligned groups of 8 lanes: on
// return, nibble r of lane c is nibble c of lane r (c = lane & 7).  Step m
// (1, 2, 4) swaps, between lanes c and c ^ m, the nibbles whose index bit m
// differs from the lane's own bit m.
__device__ __forceinline__ uint32_t nib_transpose8(uint32_t x, int c) {
    constexpr uint32_t kKeep[3] = {0x0F0F0F0Fu, 0x00FF00FFu, 0x0000FFFFu};  // nibbles with index bit m clear
#pragma unroll
    for (int s = 0; s < 3; ++s) {
        const int m = 1 << s, sh = 4 << s;
        const uint32_t y = __shfl_xor_sync(0xffffffffu, x, m);
        x = (c & m) ? ((x & ~kKeep[s]) | ((y >> sh) & kKeep[s])) : ((x & kKeep[s]) | ((y << sh) & ~kKeep[s]));
    }
    return x;
}

// ---- block reductions -------------------------------------------------------
__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

__device__ __forceinline__ float warp_sum_f(float v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// Per-thread FP32 sums a, b reduced in FP32 within each warp and in FP64
// across warps; results valid in thread 0.  scratch >= 2*32 doubles.
__device__ __forceinline__ void block_sum2_f(float a, float b, double &sa, double &sb, double *scratch) {
    a = warp_sum_f(a);
    b = warp_sum_f(b);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int nw = (blockDim.x + 31) >> 5;
    __syncthreads();
    if (lane == 0) {
        scratch[warp] = a;
        scratch[32 + warp] = b;
    }
    __syncthreads();
    sa = 0.0;
    sb = 0.0;
    if (threadIdx.x == 0)
        for (int w = 0; w < nw; ++w) {
            sa += scratch[w];
            sb += scratch[32 + w];
        }
}

// Sums a and b over the block; result valid in thread 0.  scratch >= 2*32 doubles.
__device__ __forceinline__ void block_sum2(double &a, double &b, double *scratch) {
    a = warp_sum(a);
    b = warp_sum(b);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int nw = (blockDim.x + 31) >> 5;
    __syncthreads();
    if (lane == 0) {
        scratch[warp] = a;
        scratch[32 + warp] = b;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        double sa = 0.0, sb = 0.0;
        for (int w = 0; w < nw; ++w) {
            sa += scratch[w];
            sb += scratch[32 + w];
        }
        a = sa;
        b = sb;
    }
}

// Packed nibble k -> (real, imag) = codes - 2.  A 2-bit code c placed in the
// mantissa of 1.5 * 2^23 gives the float 12582912 + c exactly; subtracting
// 12582914 leaves c - 2 (one logic op and one add, no int-to-float convert).
__device__ __forceinline__ float2 nib_value(const uint32_t *sp, int k) {
    const uint32_t w = sp[k >> 3] >> ((k & 7) * 4);
    const float re = __uint_as_float(0x4B400000u | ((w >> 2) & 3u)) - 12582914.0f;
    const float im = __uint_as_float(0x4B400000u | (w & 3u)) - 12582914.0f;
    return make_float2(re, im);
}

// Hermitian pair of a length-32768 C2R input: from Y[k], Y[M-k] (M = 16384)
// and we = e^{+2 pi i k/32768},
//   Z[k]   = (Y[k] + conj Y[M-k]) + i we (Y[k] - conj Y[M-k]) =: e + i t
//   Z[M-k] = conj(e) + i conj(t),
// so one complex multiply serves both.
__device__ __forceinline__ void c2r_pair(float2 y, float2 ym, float2 we, float2 &zk, float2 &zmk) {
    const float2 e = make_float2(y.x + ym.x, y.y - ym.y);
    const float2 t = cmul(make_float2(y.x - ym.x, y.y + ym.y), we);
    zk = make_float2(e.x - t.y, e.y + t.x);
    zmk = make_float2(e.x + t.y, t.x - e.y);
}

// Hermitian pair of a length-36608 R2C output: from Z[q], Z[M'-q] (M' = 18304)
// and w = e^{-2 pi i q/36608}, with s = Z[q] + conj Z[M'-q], t = w (Z[q] - conj Z[M'-q]):
//   X[q] = (s - i t)/2,   X[M'-q] = (conj(s) - i conj(t))/2.
__device__ __forceinline__ void r2c_pair(float2 za, float2 zb, float2 w, float2 &xq, float2 &xmq) {
    const float2 s = make_float2(za.x + zb.x, za.y - zb.y);
    const float2 t = cmul(w, make_float2(za.x - zb.x, za.y + zb.y));
    xq = make_float2(0.5f * (s.x + t.y), 0.5f * (s.y - t.x));
    xmq = make_float2(0.5f * (s.x - t.y), -0.5f * (s.y + t.x));
}


}  // namespace sdbe
