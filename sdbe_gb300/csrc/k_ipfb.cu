// Inverse polyphase filter bank for PFB-mode SWARM spectra: Shaw's
// least-squares inversion, the method of
// software/prototyping/cuda/pfb_inverse.cu:213-488.
//
// The forward PFB (pfb_inverse.cu:173-207) maps ntap consecutive time blocks
// x_i..x_{i+ntap-1} of L = 32768 samples to the spectrum S_i whose C2R is
// y_i[p] = sum_t w[t*L + p] x_{i+t}[p] (w: Hamming over ntap*L, :51-53).  For
// each phase p that is y[:, p] = P_p x[:, p] with P_p banded (nblock x
// nblock+ntap-1); the inverse is x = P^T (P P^T)^-1 y, P P^T symmetric banded
// Toeplitz with a[d] = sum_k w[(k+d)L + p] w[kL + p].
//
// GB300 layout: the pseudo time stream comes from the complex-input C2R
// kernel (one CTA per snapshot, smem-resident 16384-point transform); the
// solve runs one thread per phase p, all of a block's phases reading
// consecutive words of each row (coalesced), walking the rows in FP64: the
// matrices are ill-conditioned (condition ~3e5 at 128 blocks, growing with
// the square of the block count), so FP32 elimination would lose the answer.
// LDL^T factor rows are formed on the fly in the forward sweep (no division
// but one per row) and streamed to scratch with the forward-substituted
// values; the backward sweep reads them once, and emits x_{m+ntap-1} as soon
// as z_m is known (the projection P^T z fused in).
#include <cuda_runtime.h>

#include <cmath>
#include <vector>

#include "handle.cuh"

namespace sdbe {

// scr layout: [nblock][NT][L]: entries 0..NT-2 = L[m][m-1-k], entry NT-1 = v_m.
template <int NT>
__global__ void __launch_bounds__(128) k_ipfb_solve(const float *__restrict__ y, int64_t nblock, double scale,
                                                    const double *__restrict__ tab, double *__restrict__ scr,
                                                    float *__restrict__ out) {
    constexpr int B = NT - 1;
    constexpr int L = kNA;
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= L) return;
    double a[NT], w[NT];
#pragma unroll
    for (int d = 0; d < NT; ++d) {
        a[d] = tab[d * L + p];
        w[d] = tab[(NT + d) * L + p];
    }
    // rows m-1..m-B of the factorisation: pl[k-1][q-1] = L[m-k][m-k-q], pd = d, pdi = 1/d, pw = forward values
    double pl[B][B], pd[B], pdi[B], pw[B];
#pragma unroll
    for (int k = 0; k < B; ++k) {
        pd[k] = 1.0;
        pdi[k] = 0.0;
        pw[k] = 0.0;
#pragma unroll
        for (int q = 0; q < B; ++q) pl[k][q] = 0.0;
    }
    for (int64_t m = 0; m < nblock; ++m) {
        double l[B];  // l[k-1] = L[m][m-k]
#pragma unroll
        for (int k = B; k >= 1; --k) {
            double s = a[k];
#pragma unroll
            for (int q = k + 1; q <= B; ++q) s -= l[q - 1] * pd[q - 1] * pl[k - 1][q - k - 1];
            l[k - 1] = m - k >= 0 ? s * pdi[k - 1] : 0.0;
        }
        double dm = a[0], wm = static_cast<double>(__ldg(y + m * L + p)) * scale;
#pragma unroll
        for (int k = 1; k <= B; ++k) {
            dm -= l[k - 1] * l[k - 1] * pd[k - 1];
            wm -= l[k - 1] * pw[k - 1];
        }
        const double dinv = 1.0 / dm;
        double *row = scr + m * NT * L + p;
#pragma unroll
        for (int k = 0; k < B; ++k) row[k * L] = l[k];
        row[B * L] = wm * dinv;
#pragma unroll
        for (int k = B - 1; k >= 1; --k) {
            pd[k] = pd[k - 1];
            pdi[k] = pdi[k - 1];
            pw[k] = pw[k - 1];
#pragma unroll
            for (int q = 0; q < B; ++q) pl[k][q] = pl[k - 1][q];
        }
        pd[0] = dm;
        pdi[0] = dinv;
        pw[0] = wm;
#pragma unroll
        for (int q = 0; q < B; ++q) pl[0][q] = l[q];
    }
    // backward sweep: z_m = v_m - sum_k L[m+k][m] z_{m+k}; rows m+1..m+B held in nl/nz
    double nl[B][B], nz[B];  // nl[k-1][q-1] = L[m+k][m+k-q]
#pragma unroll
    for (int k = 0; k < B; ++k) {
        nz[k] = 0.0;
#pragma unroll
        for (int q = 0; q < B; ++q) nl[k][q] = 0.0;
    }
    for (int64_t m = nblock - 1; m >= 0; --m) {
        const double *row = scr + m * NT * L + p;
        double z = row[B * L];
#pragma unroll
        for (int k = 1; k <= B; ++k) z -= nl[k - 1][k - 1] * nz[k - 1];
        // x_{m+B} = sum_t w[t] z_{m+B-t}, t = 0..B  (z_{m..m+B} known)
        double x = w[B] * z;
#pragma unroll
        for (int t = 0; t < B; ++t) x += w[t] * nz[B - 1 - t];
        out[(m + B) * L + p] = static_cast<float>(x);
#pragma unroll
        for (int k = B - 1; k >= 1; --k) {
            nz[k] = nz[k - 1];
#pragma unroll
            for (int q = 0; q < B; ++q) nl[k][q] = nl[k - 1][q];
        }
        nz[0] = z;
#pragma unroll
        for (int q = 0; q < B; ++q) nl[0][q] = row[q * L];
    }
    // x_j for j = B-1 .. 0: z_0..z_{B-1} are nz[0..B-1]
#pragma unroll
    for (int j = B - 1; j >= 0; --j) {
        double x = 0.0;
#pragma unroll
        for (int t = 0; t <= j; ++t) x += w[t] * nz[j - t];
        out[j * L + p] = static_cast<float>(x);
    }
}

namespace {

// Host table per ntap: a[d][p] (band of P P^T) and w[t][p] (P taps), FP64.
std::vector<double> ipfb_table(int ntap) {
    const int L = kNA;
    const double m = static_cast<double>(ntap) * L;
    std::vector<double> win(static_cast<size_t>(ntap) * L);
    for (int64_t n = 0; n < static_cast<int64_t>(win.size()); ++n)
        win[n] = 0.54 - 0.46 * std::cos(2.0 * 3.14159265358979323846 * static_cast<double>(n) / (m - 1.0));
    std::vector<double> tab(static_cast<size_t>(2) * ntap * L);
    for (int d = 0; d < ntap; ++d)
        for (int p = 0; p < L; ++p) {
            double s = 0.0;
            for (int k = 0; k < ntap - d; ++k) s += win[static_cast<size_t>(k + d) * L + p] * win[static_cast<size_t>(k) * L + p];
            tab[static_cast<size_t>(d) * L + p] = s;
            tab[static_cast<size_t>(ntap + d) * L + p] = win[static_cast<size_t>(d) * L + p];
        }
    return tab;
}

template <int NT>
cudaError_t launch_solve(const float *y, int64_t nblock, const double *tab, double *scr, float *out, cudaStream_t st) {
    k_ipfb_solve<NT><<<kNA / 128, 128, 0, st>>>(y, nblock, 1.0 / kNA, tab, scr, out);
    return cudaGetLastError();
}

}  // namespace
}  // namespace sdbe

using namespace sdbe;

extern "C" int sdbe_inverse_pfb(sdbe_resampler *h, const void *spec_c64, int64_t nblock, int32_t ntap, float *out,
                                void *stream) {
    if (!h || nblock < 1 || ntap < 2 || ntap > 8 || !spec_c64 || !out) return fail(h, SDBE_ERR_ARG, "bad argument");
    if (reinterpret_cast<uintptr_t>(spec_c64) & 7u)  // read as float2
        return fail(h, SDBE_ERR_ARG, "complex spectra must be 8-byte aligned");
    if (nblock > (int64_t(1) << 20)) return fail(h, SDBE_ERR_CAPACITY, "at most 2^20 blocks per call");
    DeviceGuard g(h->cfg.device);
    if (!g.ok) return fail(h, SDBE_ERR_CUDA, "cudaSetDevice failed");
    cudaStream_t st = stream ? static_cast<cudaStream_t>(stream) : h->stream;
    if (h->ipfb_ntap != ntap) {
        const std::vector<double> tab = ipfb_table(ntap);
        if (h->ipfb_tab) {
            SDBE_CK(h, cudaDeviceSynchronize());
            cudaFree(h->ipfb_tab);
            h->ipfb_tab = nullptr;
            h->ipfb_ntap = 0;
        }
        SDBE_CK(h, cudaMalloc(&h->ipfb_tab, tab.size() * sizeof(double)));
        SDBE_CK(h, cudaMemcpyAsync(h->ipfb_tab, tab.data(), tab.size() * sizeof(double), cudaMemcpyHostToDevice, st));
        SDBE_CK(h, cudaStreamSynchronize(st));  // tab is freed on return
        h->ipfb_ntap = ntap;
    }
    // scratch owned by the handle, grown to the largest call so far
    if (int rc = grow(h, &h->ipfb_y, &h->ipfb_y_bytes, nblock * kNA * static_cast<int64_t>(sizeof(float)),
                      "the inverse PFB scratch"))
        return rc;
    if (int rc = grow(h, &h->ipfb_scr, &h->ipfb_scr_bytes,
                      nblock * ntap * kNA * static_cast<int64_t>(sizeof(double)), "the inverse PFB scratch"))
        return rc;
    float *y = reinterpret_cast<float *>(h->ipfb_y);
    double *scr = reinterpret_cast<double *>(h->ipfb_scr);
    cudaError_t e = cudaSuccess;
    if (h->cfg.precision != SDBE_PRECISION_FP32) {
        // the pseudo time stream on the tensor cores; scr holds the paired spectra
        // first (n x 16384 complex fits its n x ntap x 32768 doubles)
        if (int rc = tc_c2r_spectra(h, static_cast<const float2 *>(spec_c64), kMA + 1, nblock,
                                    reinterpret_cast<float2 *>(scr), y, st))
            return rc;
    } else {
        e = launch_r2dbe_c2r(spec_c64, kMA + 1, nblock, 0, y, h->tw, st);
    }
    if (e == cudaSuccess) {
        switch (ntap) {
            case 2: e = launch_solve<2>(y, nblock, h->ipfb_tab, scr, out, st); break;
            case 3: e = launch_solve<3>(y, nblock, h->ipfb_tab, scr, out, st); break;
            case 4: e = launch_solve<4>(y, nblock, h->ipfb_tab, scr, out, st); break;
            case 5: e = launch_solve<5>(y, nblock, h->ipfb_tab, scr, out, st); break;
            case 6: e = launch_solve<6>(y, nblock, h->ipfb_tab, scr, out, st); break;
            case 7: e = launch_solve<7>(y, nblock, h->ipfb_tab, scr, out, st); break;
            default: e = launch_solve<8>(y, nblock, h->ipfb_tab, scr, out, st); break;
        }
    }
    if (e != cudaSuccess) return fail(h, SDBE_ERR_CUDA, std::string("inverse_pfb: ") + cudaGetErrorString(e));
    h->launches += 2;
    return SDBE_OK;
}
