// df.cu — frequency-shift images from Fz stacks on the GPU.
//
// The reference turns the scan files into frequency-shift images with its
// post-processing script (simple-vafm-image.py:77-89, 204), Giessibl's
// small-amplitude formula: for every window of nosc consecutive heights
//   df(x, y) = -fshiftfac * dz * sum_m W[m] * Fz(x, y, z_m),
//   fshiftfac = f0 / (2 k) * 2 / (pi A^2),   W(z) = z / sqrt(|A^2 - z^2|)
// on the offsets z = (-zosc[L-1], ..., -zosc[2], zosc[0], ..., zosc[L-1])
// with zosc = 0, dz, 2 dz, ... (L = ceil((A + dz) / dz) values, numpy's
// arange), both end points dropped.  Heights are taken in ascending z (the
// script sorts the scan file names); window s covers heights s .. s+nosc-1.
// The operator is linear in Fz, so its adjoint is the transposed sum
// (mafm_df_adjoint), used to take gradients of a loss on df images.
#include <cmath>
#include <vector>

#include "mafm_internal.h"

namespace mafm {
namespace {

constexpr int kMaxW = 4096;

// Python's float floor division and modulo (the script's `//` and `%`):
// both go through fmod, so 0.5 // 0.1 is 4.0 although floor(0.5 / 0.1) is 5.
double py_floordiv(double a, double b) {
    double mod = std::fmod(a, b);
    double div = (a - mod) / b;
    if (mod != 0 && ((b < 0) != (mod < 0))) div -= 1.0;
    if (div != 0) {
        double f = std::floor(div);
        if (div - f > 0.5) f += 1.0;
        return f;
    }
    return std::copysign(0.0, a / b);
}

double py_mod(double a, double b) {
    double mod = std::fmod(a, b);
    if (mod != 0) {
        if ((b < 0) != (mod < 0)) mod += b;
    } else {
        mod = std::copysign(0.0, b);
    }
    return mod;
}

// Weights and prefactor exactly as the script builds them.
void df_weights(const mafm_df_params& prm, double dz, std::vector<double>& w, double& fac) {
    double amplitude = prm.amplitude;
    const double k = prm.k_cantilever, f0 = prm.f0;
    fac = (f0 / (2 * k)) * (2 / (3.14159265358979323846 * amplitude * amplitude));
    // ampcut = (1+(amplitude/dz))%(1+(amplitude//dz)): W is infinite at +-A
    const double ampcut = py_mod(1 + (amplitude / dz), 1 + py_floordiv(amplitude, dz));
    if (ampcut < 0.01) amplitude += dz / 2;
    const double stop = amplitude + dz;
    const long long L = (long long)std::ceil((stop - 0.0) / dz);
    if (L < 3 || L > kMaxW) fail(MAFM_E_RANGE, "frequency-shift window of %lld heights", L);
    std::vector<double> zosc((size_t)L);
    for (long long i = 0; i < L; ++i) zosc[i] = 0.0 + i * dz;
    std::vector<double> full;
    for (long long i = L - 1; i > 1; --i) full.push_back(-zosc[i]);
    for (long long i = 0; i < L; ++i) full.push_back(zosc[i]);
    w.clear();
    for (size_t i = 1; i + 1 < full.size(); ++i) {
        const double z = full[i];
        w.push_back(z / std::sqrt(std::fabs(amplitude * amplitude - z * z)));
    }
}

// One thread per (window, x, y): out[s][x][y].  fz is read with a stride (in
// doubles) so that it can be the force[2] field of mafm_point records.
__global__ void df_kernel(const double* fz, long long stride, int nx, int ny, int nz,
                          const double* w, int nosc, double scale, double* out, int nshift) {
    const long long tid = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const long long total = (long long)nshift * nx * ny;
    if (tid >= total) return;
    const int s = (int)(tid / ((long long)nx * ny));
    const long long xy = tid % ((long long)nx * ny);
    double acc = 0;
    for (int m = 0; m < nosc; ++m) {
        const int h = s + m;                 // ascending-z height index
        const int k = nz - 1 - h;            // scan level (k = 0 is zhigh)
        acc += w[m] * fz[(xy * nz + k) * stride];
    }
    out[tid] = -scale * acc;
}

// Transpose: g_fz[x][y][k] = -scale * sum_{s,m: s+m = nz-1-k} w[m] g_df[s][x][y].
__global__ void df_adjoint_kernel(const double* gdf, int nx, int ny, int nz, const double* w,
                                  int nosc, double scale, double* gfz, int nshift) {
    const long long tid = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const long long total = (long long)nx * ny * nz;
    if (tid >= total) return;
    const int k = (int)(tid % nz);
    const long long xy = tid / nz;
    const int h = nz - 1 - k;
    double acc = 0;
    for (int m = 0; m < nosc; ++m) {
        const int s = h - m;
        if (s >= 0 && s < nshift) acc += w[m] * gdf[(long long)s * nx * ny + xy];
    }
    gfz[tid] = -scale * acc;
}

bool dev_ptr(const void* p) {
    cudaPointerAttributes a{};
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    return a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged;
}

mafm_df_params defaults(const mafm_df_params* p) {
    if (p) return *p;
    mafm_df_params d;
    d.amplitude = 0.50;                 // simple-vafm-image.py:78
    d.k_cantilever = 1800 * 1.438978;   // :79 (N/m in kcal/mol/A^2)
    d.f0 = 25.000e3;                    // :80
    return d;
}

}  // namespace
}  // namespace mafm

using namespace mafm;

extern "C" int mafm_df_weights(const mafm_df_params* params, double dz, double* w, int32_t cap,
                               int32_t* n_w, double* fshiftfac) {
    return guarded([&] {
        if (dz <= 0) fail(MAFM_E_INVALID, "dz must be positive");
        std::vector<double> ww;
        double fac;
        df_weights(defaults(params), dz, ww, fac);
        if (n_w) *n_w = (int32_t)ww.size();
        if (fshiftfac) *fshiftfac = fac;
        if (w) {
            if (cap < (int32_t)ww.size()) fail(MAFM_E_RANGE, "weight buffer of %d < %zu", cap, ww.size());
            for (size_t i = 0; i < ww.size(); ++i) w[i] = ww[i];
        }
    });
}

// Shared by mafm_df and mafm_df_adjoint: host or device buffers, one stream.
static int df_apply(bool adjoint, const double* in, int64_t stride, int32_t nx, int32_t ny, int32_t nz,
                    double dz, const mafm_df_params* params, double* out, void* stream) {
    return guarded([&] {
        if (!in || !out || nx < 1 || ny < 1 || nz < 1) fail(MAFM_E_INVALID, "bad df arguments");
        std::vector<double> ww;
        double fac;
        df_weights(defaults(params), dz, ww, fac);
        const int nosc = (int)ww.size();
        const int nshift = nz - nosc;
        if (nshift <= 0) fail(MAFM_E_RANGE, "%d heights are fewer than the %d-height window", nz, nosc);
        cudaStream_t st = (cudaStream_t)stream;
        const long long nfz = (long long)nx * ny * nz, ndf = (long long)nshift * nx * ny;
        const long long n_in = adjoint ? ndf : (nfz - 1) * (stride > 0 ? stride : 1) + 1;
        const long long n_out = adjoint ? nfz : ndf;
        double *din = nullptr, *dout = nullptr, *dw = nullptr;
        struct Frees {
            std::vector<void*> p;
            ~Frees() { for (void* q : p) cudaFree(q); }
        } frees;
        auto dalloc = [&](double** p, long long n) {
            cuda_check(cudaMalloc(p, (size_t)n * sizeof(double)), "cudaMalloc");
            frees.p.push_back(*p);
        };
        const double* src = in;
        if (!dev_ptr(in)) {
            dalloc(&din, n_in);
            cuda_check(cudaMemcpyAsync(din, in, (size_t)n_in * sizeof(double), cudaMemcpyHostToDevice, st), "upload");
            src = din;
        }
        const bool host_out = !dev_ptr(out);
        double* dst = out;
        if (host_out) {
            dalloc(&dout, n_out);
            dst = dout;
        }
        dalloc(&dw, nosc);
        cuda_check(cudaMemcpyAsync(dw, ww.data(), nosc * sizeof(double), cudaMemcpyHostToDevice, st), "upload");
        const double scale = fac * dz;
        const unsigned blocks = (unsigned)((n_out + 255) / 256);
        if (adjoint) df_adjoint_kernel<<<blocks, 256, 0, st>>>(src, nx, ny, nz, dw, nosc, scale, dst, nshift);
        else df_kernel<<<blocks, 256, 0, st>>>(src, stride > 0 ? stride : 1, nx, ny, nz, dw, nosc, scale, dst, nshift);
        cuda_check(cudaGetLastError(), "df launch");
        if (host_out)
            cuda_check(cudaMemcpyAsync(out, dst, (size_t)n_out * sizeof(double), cudaMemcpyDeviceToHost, st), "download");
        cuda_check(cudaStreamSynchronize(st), "df");
    });
}

extern "C" int mafm_df(const double* fz, int64_t stride, int32_t nx, int32_t ny, int32_t nz, double dz,
                       const mafm_df_params* params, double* df, void* stream) {
    return df_apply(false, fz, stride, nx, ny, nz, dz, params, df, stream);
}

extern "C" int mafm_df_adjoint(const double* g_df, int32_t nx, int32_t ny, int32_t nz, double dz,
                               const mafm_df_params* params, double* g_fz, void* stream) {
    return df_apply(true, g_df, 1, nx, ny, nz, dz, params, g_fz, stream);
}
