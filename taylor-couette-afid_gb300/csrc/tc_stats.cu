// tc_stats.cu -- the statistics of the reference's output steps on the
// device: CalcStats (StatRoutines.F90:13-76, with CalcVorticity.F90:30-70)
// and CalcDissipation (CalcDissipation.F90:22-74).
//
// Both accumulate theta averages per (r, z) row into FP64 arrays kept in the
// handle (the reference's stat_arrays, (nrm, nzm), r fastest).  One warp per
// row: the lanes stride over theta, keep FP64 partial sums of every
// statistic, and reduce them with shuffles; the row's sums are then added to
// the arrays by one lane, so every array entry has one writer.  The volume
// integral of the dissipation is summed per row and then over the rows by
// one block in a fixed order, so it is deterministic.  The mixed form reads
// its FP32 fields and reduces in FP64.
//
// Reference quirks kept: CalcStats takes the clamped kpv(k) as the radial
// neighbour of its correlations and sums qz(k,j,i) + qr(k,j+1,i) in
// vtvz_mean (StatRoutines.F90:58); udx2mm(nrm) uses rm(nr), which CreateGrid
// never sets (0).

#include <string>

#include "tc_bodies.cuh"
#include "tc_handle.h"

namespace tcgb {
void set_last_error(const std::string& msg);

namespace stats {

constexpr int kWarps = 8;   // rows per block

__device__ __forceinline__ double dv(const double* p, size_t o) { return __ldg(p + o); }
__device__ __forceinline__ double dv(const float* p, size_t o) { return f2d(__ldg(p + o)); }

__device__ __forceinline__ double wsum(double v) {
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

template <typename T>
__global__ void __launch_bounds__(32 * kWarps) stats_kernel(Dims d, Coef c, Consts kc, FieldsT<T> f, double* st,
                                                            double* rows, int do_stats, int do_diss) {
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const long long row = (long long)blockIdx.x * kWarps + warp;
    const int nrm = d.nr, nzm = d.nz, nt = d.nt;
    if (row >= (long long)nrm * nzm) return;
    const int k = (int)(row % nrm), j = (int)(row / nrm);      // 0-based; reference k+1, j+1
    const size_t P = (size_t)d.P;
    const int kpv = k < nrm - 1 ? k + 1 : nrm - 1, kmv = k > 0 ? k - 1 : 0, kp = k + 1;
    const int jm = j == 0 ? nzm - 1 : j - 1, jp = j == nzm - 1 ? 0 : j + 1;
    const double usnthm = 1.0 / nt;
    const double usrc = c.usrc[k], usrcp = c.usrc[kp], usrckpv = c.usrc[kpv], usrckmv = c.usrc[kmv];
    const double usrm = c.usrm[k], usrmkpv = c.usrm[kpv], usrmkmv = c.usrm[kmv];
    const double rmk = c.rm[k], rmkpv = c.rm[kpv], rmkmv = c.rm[kmv];
    const double udx2mm = c.udx2mm[k], udx2cc = c.udx2cc[k];
    const double dxt = kc.dxt, dxz = kc.dxz;
    double s[TC_ST_COUNT];
#pragma unroll
    for (int a = 0; a < TC_ST_COUNT; ++a) s[a] = 0.0;
    double diss = 0.0;
    auto at = [&](int kk, int jj, int ii) { return (size_t)kk * P + (size_t)jj * nt + ii; };
    for (int i = lane; i < nt; i += 32) {
        const int im = i == 0 ? nt - 1 : i - 1, ip = i == nt - 1 ? 0 : i + 1;
        const double qt = dv(f.qt, at(k, j, i)), qr = dv(f.qr, at(k, j, i)), qz = dv(f.qz, at(k, j, i));
        if (do_stats) {
            // CalcVorticity.F90:45-70 (kp = k+1, kpp/kmm clamped)
            const double durdz = ((dv(f.qr, at(kp, jp, i)) * usrcp + dv(f.qr, at(k, jp, i)) * usrc)
                                  - (dv(f.qr, at(kp, jm, i)) * usrcp + dv(f.qr, at(k, jm, i)) * usrc)) * dxz * 0.25;
            const double duzdr = ((dv(f.qz, at(kpv, j, i)) + dv(f.qz, at(kpv, jp, i)))
                                  - (dv(f.qz, at(kmv, j, i)) + dv(f.qz, at(kmv, jp, i)))) * 0.5 * udx2mm;
            const double wt = durdz - duzdr;
            const double duzdt = ((dv(f.qz, at(k, j, ip)) + dv(f.qz, at(k, jp, ip)))
                                  - (dv(f.qz, at(k, j, im)) + dv(f.qz, at(k, jp, im)))) * 0.25 * dxt * usrm;
            const double dutdz = ((dv(f.qt, at(k, jp, i)) + dv(f.qt, at(k, jp, ip)))
                                  - (dv(f.qt, at(k, jm, i)) + dv(f.qt, at(k, jm, ip)))) * 0.25 * dxz;
            const double wr = duzdt - dutdz;
            const double dutdr = ((dv(f.qt, at(kpv, j, i)) + dv(f.qt, at(kpv, j, ip))) * rmkpv
                                  - (dv(f.qt, at(kmv, j, i)) + dv(f.qt, at(kmv, j, ip))) * rmkmv) * 0.5 * udx2mm * usrm;
            const double durdt = ((dv(f.qr, at(k, j, ip)) * usrc + dv(f.qr, at(kp, j, ip)) * usrcp)
                                  - (dv(f.qr, at(k, j, im)) * usrc + dv(f.qr, at(kp, j, im)) * usrcp)) * dxt * 0.25;
            const double wz = dutdr - durdt;
            const double prv = f.pr[at(k, j, i)];
            // StatRoutines.F90:34-66
            s[TC_ST_VT_MEAN] += qt * usnthm;
            s[TC_ST_VR_MEAN] += qr * usnthm * usrc;
            s[TC_ST_VZ_MEAN] += qz * usnthm;
            s[TC_ST_WT_MEAN] += wt * usnthm;
            s[TC_ST_WR_MEAN] += wr * usnthm;
            s[TC_ST_WZ_MEAN] += wz * usnthm;
            s[TC_ST_VT_RMS] += qt * qt * usnthm;
            s[TC_ST_VR_RMS] += (qr * usrc) * (qr * usrc) * usnthm;
            s[TC_ST_VZ_RMS] += qz * qz * usnthm;
            s[TC_ST_WT_RMS] += wt * wt * usnthm;
            s[TC_ST_WR_RMS] += wr * wr * usnthm;
            s[TC_ST_WZ_RMS] += wz * wz * usnthm;
            s[TC_ST_PR_MEAN] += prv * usnthm;
            s[TC_ST_PR_RMS] += prv * prv * usnthm;
            const double qtip = dv(f.qt, at(k, j, ip));
            const double qrk = qr * usrc + dv(f.qr, at(kpv, j, i)) * usrckpv;
            s[TC_ST_VTVR_MEAN] += (qt + qtip) * qrk * usnthm * 0.25;
            s[TC_ST_VTVZ_MEAN] += (qt + qtip) * (qz + dv(f.qr, at(k, jp, i))) * usnthm * 0.25;
            s[TC_ST_VRVZ_MEAN] += (qz + dv(f.qz, at(k, jp, i))) * qrk * usnthm * 0.25;
        }
        if (do_diss) {
            // CalcDissipation.F90:39-58
            const double e11 = (dv(f.qt, at(k, j, ip)) - dv(f.qt, at(k, j, im))) * dxt * usrm * 0.5 + qr * (usrc * usrc);
            const double e12 = (dv(f.qt, at(kpv, j, i)) * usrmkpv - dv(f.qt, at(kmv, j, i)) * usrmkmv) * udx2mm * rmk
                               + (dv(f.qr, at(k, j, ip)) - dv(f.qr, at(k, j, im))) * usrc * dxt * 0.5;
            const double e13 = (dv(f.qt, at(k, jp, i)) - dv(f.qt, at(k, jm, i))) * 0.5 * dxz
                               + (dv(f.qz, at(k, j, ip)) - dv(f.qz, at(k, j, im))) * 0.5 * dxt * usrm;
            const double e22 = (dv(f.qr, at(kp, j, i)) * usrcp - dv(f.qr, at(kmv, j, i)) * usrckmv) * udx2cc;
            const double e23 = (dv(f.qz, at(kpv, j, i)) - dv(f.qz, at(kmv, j, i))) * udx2mm
                               + (dv(f.qr, at(k, jp, i)) - dv(f.qr, at(k, jm, i))) * usrc * dxz * 0.5;
            const double e33 = (dv(f.qz, at(k, jp, i)) - dv(f.qz, at(k, jm, i))) * dxz * 0.5;
            const double dis = 2.0 * (e11 * e11 + e22 * e22 + e33 * e33) + e12 * e12 + e13 * e13 + e23 * e23;
            diss += dis;
        }
    }
#pragma unroll
    for (int a = 0; a < TC_ST_COUNT; ++a) s[a] = wsum(s[a]);
    diss = wsum(diss);
    if (lane == 0) {
        const size_t NS = (size_t)nrm * nzm;
        if (do_stats)
            for (int a = 0; a < TC_ST_DISSTE; ++a) st[(size_t)a * NS + row] += s[a];
        if (do_diss) {
            st[(size_t)TC_ST_DISSTE * NS + row] += diss / kc.ren / (double)nt;
            rows[row] = diss * c.pvol[k] * kc.pi;
        }
    }
}

// nute = sum over rows / (nthm nzm volt lamdissip), CalcDissipation.F90:64-72
__global__ void nute_kernel(const double* rows, long long n, double den, double* out) {
    __shared__ double sh[256];
    double v = 0.0;
    for (long long t = threadIdx.x; t < n; t += blockDim.x) v += rows[t];
    sh[threadIdx.x] = v;
    __syncthreads();
    for (int o = blockDim.x / 2; o > 0; o >>= 1) {
        if ((int)threadIdx.x < o) sh[threadIdx.x] += sh[threadIdx.x + o];
        __syncthreads();
    }
    if (threadIdx.x == 0) *out = sh[0] / den;
}

int sfail(tc_handle* h, int code, const std::string& msg) {
    if (h) h->err = msg;
    set_last_error(msg);
    return code;
}

int ensure(tc_handle* h) {
    if (h->stats) return 0;
    const size_t ns = (size_t)h->d.nr * h->d.nz;
    const size_t bytes = sizeof(double) * (TC_ST_COUNT * ns + ns + 8);
    void* p = nullptr;
    cudaError_t e = cudaMalloc(&p, bytes);
    if (e == cudaSuccess) e = cudaMemsetAsync(p, 0, bytes, h->stream);
    if (e != cudaSuccess) return sfail(h, 1000 + (int)e, std::string("statistics arrays: ") + cudaGetErrorString(e));
    h->allocs.push_back(p);
    h->bytes += (long long)bytes;
    h->stats = (double*)p;
    h->stat_rows = h->stats + TC_ST_COUNT * ns;
    return 0;
}

int run(tc_handle* h, int do_stats, int do_diss, double* nute) {
    if (!h) return sfail(nullptr, 2000, "null handle");
    if (int r = ensure(h)) return r;
    const long long nrows = (long long)h->d.nr * h->d.nz;
    const unsigned blocks = (unsigned)((nrows + kWarps - 1) / kWarps);
    if (h->mixed)
        stats_kernel<float><<<blocks, 32 * kWarps, 0, h->stream>>>(h->d, h->c, h->k, h->ff, h->stats, h->stat_rows,
                                                                   do_stats, do_diss);
    else
        stats_kernel<double><<<blocks, 32 * kWarps, 0, h->stream>>>(h->d, h->c, h->k, h->fd, h->stats, h->stat_rows,
                                                                    do_stats, do_diss);
    h->launches += 1;
    if (do_stats) h->nstatsamples += 1;
    if (do_diss) {
        const tc_bou& b = h->bou;
        const double pi = h->k.pi;
        const double volt = pi * (b.rext * b.rext - b.rint * b.rint);
        const double a = (b.virotint / b.rint - b.virotext / b.rext) / (b.rext - b.rint);
        const double lamdissip = 4.0 * b.rext * b.rext * b.rint * b.rint / ((b.rext + b.rint) * (b.rext + b.rint)) * (a * a);
        const double den = (double)h->d.nt * (double)h->d.nz * volt * lamdissip;
        double* dout = h->stat_rows + nrows;
        nute_kernel<<<1, 256, 0, h->stream>>>(h->stat_rows, nrows, den, dout);
        h->launches += 1;
        double v = 0.0;
        cudaError_t e = cudaMemcpyAsync(&v, dout, sizeof v, cudaMemcpyDeviceToHost, h->stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
        if (e != cudaSuccess) return sfail(h, 1000 + (int)e, std::string("dissipation: ") + cudaGetErrorString(e));
        if (nute) *nute = v;
    }
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return sfail(h, 1000 + (int)e, std::string("statistics launch: ") + cudaGetErrorString(e));
    return 0;
}

}  // namespace stats
}  // namespace tcgb

using namespace tcgb;

// Declared extern "C" in tc_capi.h.

int tc_calc_stats(tc_handle* h) { return stats::run(h, 1, 0, nullptr); }

int tc_calc_dissipation(tc_handle* h, double* nute) { return stats::run(h, 0, 1, nute); }

int tc_get_stat(tc_handle* h, int which, double* out) {
    if (!h || !out) return stats::sfail(h, 2000, "null argument");
    if (which < 0 || which >= TC_ST_COUNT) return stats::sfail(h, 2000, "unknown statistic");
    if (int r = stats::ensure(h)) return r;
    const size_t ns = (size_t)h->d.nr * h->d.nz;
    cudaError_t e = cudaMemcpyAsync(out, h->stats + (size_t)which * ns, sizeof(double) * ns, cudaMemcpyDeviceToHost,
                                    h->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
    if (e != cudaSuccess) return stats::sfail(h, 1000 + (int)e, std::string("statistics read: ") + cudaGetErrorString(e));
    return 0;
}

int tc_stat_samples(const tc_handle* h) { return h ? h->nstatsamples : 0; }

int tc_reset_stats(tc_handle* h) {
    if (!h) return stats::sfail(nullptr, 2000, "null handle");
    h->nstatsamples = 0;
    if (!h->stats) return 0;
    const size_t ns = (size_t)h->d.nr * h->d.nz;
    cudaError_t e = cudaMemsetAsync(h->stats, 0, sizeof(double) * TC_ST_COUNT * ns, h->stream);
    if (e != cudaSuccess) return stats::sfail(h, 1000 + (int)e, std::string("statistics reset: ") + cudaGetErrorString(e));
    return 0;
}
