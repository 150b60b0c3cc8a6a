// tc_capi.cu -- the C ABI (include/tc_capi.h): handle, device memory, the
// step sequence and the per-routine entry points, for the plain FP64 path
// and the mixed FP32/FP64 path.

#include <sys/mman.h>

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <limits>
#include <map>
#include <mutex>
#include <string>
#include <type_traits>
#include <vector>

#include "../../include/tc_capi.h"
#include "tc_grid.h"
#include "tc_handle.h"
#include "tc_kernels.cuh"

using namespace tcgb;

namespace {

std::string g_last_error;

int fail(tc_handle* h, int code, const std::string& msg) {
    if (h) h->err = msg;
    g_last_error = msg;
    return code;
}

int cuda_fail(tc_handle* h, cudaError_t e, const char* what) {
    return fail(h, 1000 + (int)e, std::string(what) + ": " + cudaGetErrorString(e));
}

#define CK(call, what) do { cudaError_t e_ = (call); if (e_ != cudaSuccess) return cuda_fail(h, e_, what); } while (0)

template <typename T>
cudaError_t dalloc(tc_handle* h, T** p, size_t count) {
    void* v = nullptr;
    cudaError_t e = cudaMalloc(&v, count * sizeof(T));
    if (e != cudaSuccess) return e;
    h->allocs.push_back(v);
    h->bytes += (long long)(count * sizeof(T));
    e = cudaMemset(v, 0, count * sizeof(T));
    *p = (T*)v;
    return e;
}

// Radix plan: radix-8 stages first when r8 (the FP32 transforms, bound by
// instruction issue: fewer passes through shared memory), then 4, 2, 3, 5,
// and the primes 7, 11, 13.
// The FP64 transforms keep radix-4 stages, whose factored multiply-add
// butterflies cost the same FP64 instructions a point and level.
bool make_plan(int n, FFTPlan& P, bool r8) {
    if (n < 1 || n > 65536) return false;
    P.n = n;
    P.nstages = 0;
    int m = n;
    if (r8)
        while (m % 8 == 0 && m > 1) {
            if (P.nstages >= kMaxStages) return false;
            P.radix[P.nstages++] = 8;
            m /= 8;
        }
    for (int r : {4, 2, 3, 5, 7, 11, 13})
        while (m % r == 0 && m > 1) {
            if (P.nstages >= kMaxStages) return false;
            P.radix[P.nstages++] = r;
            m /= r;
        }
    int L = 1;
    for (int st = 0; st < P.nstages; ++st) {
        L *= P.radix[st];
        P.rp[st] = n / L;
        P.mrp[st] = div_magic((unsigned)P.rp[st]);
    }
    P.mn = div_magic((unsigned)n);
    P.mn1 = div_magic((unsigned)n + 1u);
    return m == 1;
}

// exp(-2 pi i j / n), j = 0..count-1, rounded once into the element type.
template <typename C2>
std::vector<C2> twiddles(int n, int count) {
    std::vector<C2> w(count);
    const long double tpi = 6.283185307179586476925286766559L;
    for (int j = 0; j < count; ++j) {
        long double a = tpi * (long double)j / (long double)n;
        w[j].x = (decltype(w[j].x))cosl(a);
        w[j].y = -(decltype(w[j].y))sinl(a);
    }
    return w;
}

// The plain table of length n (padded to an even count) followed by the
// factored forms of the same twiddles for the multiply-add butterflies of
// tc_fft.cuh: n entries of exp(-2 pi i j / n), then n of exp(+2 pi i j / n),
// each {g, fx, fy, swap} from the long double cosine and sine.
template <typename C2>
std::vector<C2> twiddles_with_factored(int n) {
    typedef decltype(C2().x) R;
    const int pad = (n + 1) & ~1;
    std::vector<C2> w = twiddles<C2>(n, n);
    w.resize((size_t)pad + 4 * (size_t)n);
    FTw<R>* f = reinterpret_cast<FTw<R>*>(w.data() + pad);
    const long double tpi = 6.283185307179586476925286766559L;
    for (int dir = 0; dir < 2; ++dir)
        for (int j = 0; j < n; ++j) {
            const long double a = tpi * (long double)j / (long double)n;
            const long double c = cosl(a), s = dir == 0 ? -sinl(a) : sinl(a);
            FTw<R>& e = f[(size_t)dir * n + j];
            if (fabsl(c) >= fabsl(s)) {
                e.g = (R)(s / c); e.fx = (R)c; e.fy = (R)c; e.swap = (R)0;
            } else {
                e.g = (R)(c / s); e.fx = (R)(-s); e.fy = (R)s; e.swap = (R)1;
            }
        }
    return w;
}

int check(tc_handle* h) {
    if (!h) return fail(nullptr, 2000, "null handle");
    return 0;
}

// Kernel classes reported by tc_profile_read.
enum { K_MOMENTUM = 0, K_RADIAL, K_DIVFFT, K_ZFFT, K_PTRI, K_THINV, K_CORRECT, K_CONTROL, K_REDUCE,
       K_LAYOUT, K_COUNT };
const char* const kClassNames[K_COUNT] = {"momentum", "radial_solve", "div_theta_fft", "z_fft",
                                          "pressure_tridiag", "theta_inverse_fft", "correct",
                                          "step_control", "reduction", "layout"};

cudaEvent_t next_event(tc_handle* h) {
    if (h->pool_used == h->pool.size()) {
        cudaEvent_t e;
        cudaEventCreate(&e);
        h->pool.push_back(e);
    }
    return h->pool[h->pool_used++];
}

// Enqueue `n` kernel launches of class `cls` done by `fn`, counting them and,
// when profiling, bracketing them with events on the handle's stream.
template <typename Fn>
void L(tc_handle* h, int cls, int n, Fn fn) {
    if (h->profiling) {
        cudaEvent_t a = next_event(h), b = next_event(h);
        cudaEventRecord(a, h->stream);
        fn();
        cudaEventRecord(b, h->stream);
        h->recs.push_back({cls, a, b});
    } else {
        fn();
    }
    h->launches += n;
    if (h->profiling) h->prof_n[cls] += n;
}

template <typename T> FieldsT<T>& F(tc_handle* h);
template <> FieldsT<double>& F<double>(tc_handle* h) { return h->fd; }
template <> FieldsT<float>& F<float>(tc_handle* h) { return h->ff; }
template <typename T> const CoefT<T>& CF(tc_handle* h);
template <> const CoefT<double>& CF<double>(tc_handle* h) { return h->c; }
template <> const CoefT<float>& CF<float>(tc_handle* h) { return h->cf; }
template <typename T> const PlansT<T>& PL(tc_handle* h);
template <> const PlansT<double>& PL<double>(tc_handle* h) { return h->pd; }
template <> const PlansT<float>& PL<float>(tc_handle* h) { return h->pf; }

// Allocate the velocity-side state of element type T.
template <typename T>
cudaError_t alloc_fields(tc_handle* h, FieldsT<T>& f) {
    const Dims& d = h->d;
    const int nr = d.nr, nrr = nr + 1;
    const size_t cells = (size_t)d.P * nr, faces = (size_t)d.P * nrr;
    cudaError_t ce = cudaSuccess;
#define AL(ptr, n) if (ce == cudaSuccess) ce = dalloc(h, &(ptr), (n))
    AL(f.qt, cells); AL(f.qr, faces); AL(f.qz, cells); AL(f.pr, cells); AL(f.phi, cells);
    AL(f.ru1, cells); AL(f.ru2, faces); AL(f.ru3, cells);
    AL(f.rhs_t, cells); AL(f.rhs_r, faces); AL(f.rhs_z, cells);
    AL(f.spec, (size_t)d.PS * nr);
    AL(f.F.base, MomFactorsT<T>::count(nrr));
    f.F.stride = nrr;
    AL(f.corr, kCorrCount(nrr));
    AL(f.scal, 8);
    AL(f.red, (size_t)6 * reduction_blocks());
    if (std::is_same<T, double>::value) f.prf = reinterpret_cast<T*>(f.pr);
    else AL(f.prf, cells);
    if (std::is_same<T, double>::value) {
        f.Fd.base = reinterpret_cast<double*>(f.F.base);
        f.Fd.stride = nrr;
        f.corrd = reinterpret_cast<double*>(f.corr);
        f.ws = nullptr;
    } else {
        AL(f.Fd.base, MomFactorsT<double>::count(nrr));
        f.Fd.stride = nrr;
        AL(f.corrd, kCorrCount(nrr));
        AL(f.ws, (size_t)d.PS * ptri_slots(nr));
    }
#undef AL
    return ce;
}

template <typename T>
cudaError_t upload_plans(tc_handle* h, PlansT<T>& p) {
    typedef typename V2<T>::type C2;
    const Dims& d = h->d;
    std::vector<C2> wt = twiddles_with_factored<C2>(d.M), wz = twiddles_with_factored<C2>(d.nz),
                    wr = twiddles<C2>(d.nt, d.M + 1);
    C2 *dwt = nullptr, *dwz = nullptr, *dwr = nullptr;
    cudaError_t ce = dalloc(h, &dwt, wt.size());
    if (ce == cudaSuccess) ce = dalloc(h, &dwz, wz.size());
    if (ce == cudaSuccess) ce = dalloc(h, &dwr, wr.size());
    if (ce == cudaSuccess) ce = cudaMemcpy(dwt, wt.data(), wt.size() * sizeof(C2), cudaMemcpyHostToDevice);
    if (ce == cudaSuccess) ce = cudaMemcpy(dwz, wz.data(), wz.size() * sizeof(C2), cudaMemcpyHostToDevice);
    if (ce == cudaSuccess) ce = cudaMemcpy(dwr, wr.data(), wr.size() * sizeof(C2), cudaMemcpyHostToDevice);
    p.tw_th = dwt; p.tw_z = dwz; p.twr = dwr;
    return ce;
}

template <typename T>
void set_coef_ptrs(CoefT<T>& c, const T* base, int lenK) {
    const T** cp[] = {&c.usrm, &c.usrc, &c.udx2rm, &c.udx1vis1, &c.udxt_m, &c.udxtq_m,
                      &c.rc, &c.udx2c, &c.udx1vis2, &c.udxt_c, &c.udxtq_c,
                      &c.ap1j, &c.ac1j, &c.am1j, &c.ap2je, &c.ac2je, &c.am2je,
                      &c.ap3j, &c.ac3j, &c.am3j, &c.ap2j, &c.ac2j, &c.am2j,
                      &c.udx2m, &c.rudx2c, &c.udx1qm, &c.apph, &c.acph, &c.amph,
                      &c.usrm2, &c.q_udx2rm, &c.q_usrm, &c.h_udx1vis1, &c.q_udx2c,
                      &c.q_rc_romeg, &c.rm, &c.udx2mm, &c.udx2cc, &c.pvol, &c.h_dxt_usrm, &c.h_udx2rm};
    for (int a = 0; a < kCoefArrays; ++a) *cp[a] = base + (size_t)a * lenK;
    c.ak1 = base + (size_t)kCoefArrays * lenK;
    c.ak3 = base + (size_t)(kCoefArrays + 1) * lenK;
}

}  // namespace

// Message for tc_last_error(NULL) from the other translation units.
namespace tcgb {
void set_last_error(const std::string& msg) { g_last_error = msg; }
void set_handle_error(tc_handle* h, const std::string& msg) {
    if (h) h->err = msg;
    g_last_error = msg;
}
}  // namespace tcgb

// The exported functions below are declared extern "C" in tc_capi.h, which
// gives these definitions C linkage.

const char* tc_last_error(const tc_handle* h) {
    if (h) return h->err.c_str();
    return g_last_error.c_str();
}

// cuTensorMapEncodeTiled of the driver, looked up through the runtime (the
// library links the runtime only).
typedef CUresult (*EncodeTiledFn)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                  const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                  CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);
static EncodeTiledFn encode_tiled() {
    static EncodeTiledFn fn = nullptr;
    static bool tried = false;
    if (!tried) {
        tried = true;
        void* p = nullptr;
        cudaDriverEntryPointQueryResult q = cudaDriverEntryPointSymbolNotFound;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
                cudaSuccess && q == cudaDriverEntryPointSuccess)
            fn = reinterpret_cast<EncodeTiledFn>(p);
        else
            cudaGetLastError();
    }
    return fn;
}

// A 3-D descriptor of an FP32 array [nplanes][nz][nt] with a box of `rows`
// z rows of 72 floats (the march's staged rows).
static bool march_map(CUtensorMap* m, const float* base, int nt, int nz, int nplanes, int rows) {
    EncodeTiledFn fn = encode_tiled();
    if (!fn) return false;
    const cuuint64_t dims[3] = {(cuuint64_t)nt, (cuuint64_t)nz, (cuuint64_t)nplanes};
    const cuuint64_t strides[2] = {(cuuint64_t)nt * 4, (cuuint64_t)nt * nz * 4};
    const cuuint32_t box[3] = {72, (cuuint32_t)rows, 1}, estr[3] = {1, 1, 1};
    return fn(m, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3, const_cast<float*>(base), dims, strides, box, estr,
              CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
              CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

// Descriptors of the mixed march for grids whose rows meet the TMA rules
// (nthm a multiple of 4, so rows start on 16-byte boundaries; nthm >= 64).
static bool make_march_maps(tc_handle* h) {
    const Dims& d = h->d;
    if (!h->mixed || d.nt % 4 != 0 || d.nt < 64) return false;
    const FieldsT<float>& f = h->ff;
    MarchMaps& M = h->maps;
    const float* q[4] = {f.qt, f.qr, f.qz, f.prf};
    const int nq[4] = {d.nr, d.nr + 1, d.nr, d.nr};
    const float* ru[3] = {f.ru1, f.ru2, f.ru3};
    const int nru[3] = {d.nr, d.nr + 1, d.nr};
    for (int c = 0; c < 4; ++c)
        if (!march_map(&M.q6[c], q[c], d.nt, d.nz, nq[c], 6) || !march_map(&M.q1[c], q[c], d.nt, d.nz, nq[c], 1))
            return false;
    for (int c = 0; c < 3; ++c)
        if (!march_map(&M.ru[c], ru[c], d.nt, d.nz, nru[c], 4)) return false;
    return true;
}

int tc_create_ex(const tc_bou* cfg, int precision, tc_handle** out) {
    if (!cfg || !out) return fail(nullptr, 2000, "null argument");
    if (precision != TC_PREC_FP64 && precision != TC_PREC_MIXED && precision != TC_PREC_MIXED_FF)
        return fail(nullptr, 2007, "unknown precision");
    *out = nullptr;
    tc_handle* h = new tc_handle();
    h->bou = *cfg;
    h->mixed = precision != TC_PREC_FP64;
    h->ptri_ff = precision == TC_PREC_MIXED_FF;
    std::string e = build_grid(*cfg, h->g);
    if (!e.empty()) { int r = fail(nullptr, 2003, e); delete h; return r; }
    int dev = 0;
    cudaError_t ce = cudaGetDevice(&dev);
    if (ce != cudaSuccess) { int r = cuda_fail(nullptr, ce, "no CUDA device"); delete h; return r; }

    const Grid& g = h->g;
    Dims& d = h->d;
    d.nt = cfg->nthm; d.nz = cfg->nzm; d.nr = cfg->nrm;
    d.M = d.nt / 2; d.PH = d.M + 1; d.nzh = d.nz / 2 + 1;
    d.P = (long long)d.nz * d.nt;
    d.PS = (long long)d.nz * d.PH;
    d.mnz = ((unsigned long long)d.nr * d.nz * d.nz < (1ull << 32)) ? div_magic((unsigned)d.nz) : 0u;
    const int nr = d.nr, nrr = nr + 1;

    Consts& k = h->k;
    std::memset(&k, 0, sizeof k);
    k.dxt = g.dxt; k.dxz = g.dxz; k.dxtq = g.dxtq; k.dxzq = g.dxzq;
    k.ren = cfg->ren; k.romeg = cfg->romeg; k.virotint = cfg->virotint; k.virotext = cfg->virotext;
    k.ap1j_fs0 = g.ap1j_fs[0]; k.ac1j_fs0 = g.ac1j_fs[0]; k.am1j_fs0 = g.am1j_fs[0];
    k.ap1j_fs1 = g.ap1j_fs[1]; k.ac1j_fs1 = g.ac1j_fs[1];
    k.ap3j_fs0 = g.ap3j_fs[0]; k.ac3j_fs0 = g.ac3j_fs[0]; k.am3j_fs0 = g.am3j_fs[0];
    k.ap3j_fs1 = g.ap3j_fs[1]; k.ac3j_fs1 = g.ac3j_fs[1];
    k.sizepert = cfg->sizepert; k.omegapert = cfg->omegapert; k.pi = g.pi;
    k.rint = cfg->rint; k.rext = cfg->rext; k.lamb = cfg->lamb;
    k.dtmin = cfg->dtmin; k.dtmax = cfg->dtmax; k.limitCFL = cfg->limitCFL; k.tout = cfg->tout;
    k.tmax = cfg->tmax; k.limitVel = cfg->limitVel; k.resid = cfg->resid;
    time_march_scheme(cfg->nsst, k.gam, k.rom, k.alm);
    k.udxz = g.dxz * 0.25;
    k.udxzq = g.dxzq / cfg->ren;
    k.q_romeg = 0.25 * cfg->romeg;
    for (int s = 0; s < 3; ++s) {
        k.alre[s] = k.alm[s] / cfg->ren;
        k.dxz_al[s] = g.dxz * k.alm[s];
        k.dxt_al[s] = g.dxt * k.alm[s];
    }
    k.fft_norm = 0.5 / ((double)cfg->nthm * (double)cfg->nzm);
    k.nsst = cfg->nsst; k.idtv = cfg->idtv; k.ntst = cfg->ntst;
    k.minstrt = cfg->minstrt; k.minstrz = cfg->minstrz; k.multmin = cfg->multmin;
    k.patterned = (cfg->minstrt * cfg->multmin + cfg->minstrz * cfg->multmin) != 0;

    // 1-D coefficient arrays, each padded to lenK entries
    std::vector<const std::vector<double>*> src = {
        &g.usrm, &g.usrc, &g.udx2rm, &g.udx1vis1, nullptr, nullptr,
        &g.rc, &g.udx2c, &g.udx1vis2, nullptr, nullptr,
        &g.ap1j, &g.ac1j, &g.am1j, &g.ap2je, &g.ac2je, &g.am2je, &g.ap3j, &g.ac3j, &g.am3j,
        &g.ap2j, &g.ac2j, &g.am2j,
        &g.udx2m, &g.rudx2c, &g.udx1qm, &g.apph, &g.acph, &g.amph, nullptr,
        nullptr, nullptr, nullptr, nullptr, nullptr,
        &g.rm, &g.udx2mm, &g.udx2cc, &g.pvol, nullptr, nullptr};
    const int lenK = std::max(std::max(nrr, d.nt), d.nz) + 1;
    std::vector<double> host((size_t)(kCoefArrays + 2) * lenK, 0.0);
    for (int a = 0; a < kCoefArrays; ++a) {
        double* dst = host.data() + (size_t)a * lenK;
        if (src[a]) for (size_t m = 0; m < src[a]->size(); ++m) dst[m] = (*src[a])[m];
    }
    for (int m = 0; m < nrr; ++m) {
        double rm = g.rm[m], rc = g.rc[m];
        host[(size_t)4 * lenK + m] = m < nr ? g.dxt * 0.25 * g.usrm[m] : 0.0;              // udxt_m
        host[(size_t)5 * lenK + m] = m < nr ? g.dxtq / (cfg->ren * (rm * rm)) : 0.0;       // udxtq_m
        host[(size_t)9 * lenK + m] = g.dxt * 0.25 * g.usrc[m];                             // udxt_c
        host[(size_t)10 * lenK + m] = g.dxtq / (cfg->ren * (rc * rc));                      // udxtq_c
        host[(size_t)29 * lenK + m] = g.usrm[m] * g.usrm[m];                                // usrm2
        host[(size_t)30 * lenK + m] = 0.25 * g.udx2rm[m];
        host[(size_t)31 * lenK + m] = 0.25 * g.usrm[m];
        host[(size_t)32 * lenK + m] = 0.5 * g.udx1vis1[m];
        host[(size_t)33 * lenK + m] = 0.25 * g.udx2c[m];
        host[(size_t)34 * lenK + m] = 0.25 * g.rc[m] * cfg->romeg;
        host[(size_t)39 * lenK + m] = m < nr ? 0.5 * g.dxt * g.usrm[m] : 0.0;                 // h_dxt_usrm
        host[(size_t)40 * lenK + m] = 0.5 * g.udx2rm[m];                                       // h_udx2rm
    }
    for (int i = 0; i < d.nt; ++i) host[(size_t)kCoefArrays * lenK + i] = g.ak1[i];
    for (int j = 0; j < d.nz; ++j) host[(size_t)(kCoefArrays + 1) * lenK + j] = g.ak3[j];
    double* dcoef = nullptr;
    ce = dalloc(h, &dcoef, host.size());
    if (ce == cudaSuccess) ce = cudaMemcpy(dcoef, host.data(), host.size() * sizeof(double), cudaMemcpyHostToDevice);
    if (ce != cudaSuccess) { int r = cuda_fail(nullptr, ce, "coefficient upload"); tc_destroy(h); return r; }
    set_coef_ptrs(h->c, (const double*)dcoef, lenK);
    if (h->mixed) {
        std::vector<float> hostf(host.size());
        for (size_t m = 0; m < host.size(); ++m) hostf[m] = (float)host[m];
        float* fcoef = nullptr;
        ce = dalloc(h, &fcoef, hostf.size());
        if (ce == cudaSuccess) ce = cudaMemcpy(fcoef, hostf.data(), hostf.size() * sizeof(float), cudaMemcpyHostToDevice);
        if (ce != cudaSuccess) { int r = cuda_fail(nullptr, ce, "coefficient upload"); tc_destroy(h); return r; }
        set_coef_ptrs(h->cf, (const float*)fcoef, lenK);
    }

    // state shared by both paths
    double *pl = nullptr, *pdv = nullptr;
    signed char* icyl = nullptr;
    ce = dalloc(h, &pl, (size_t)d.nzh * d.PH * nr);
    if (ce == cudaSuccess) ce = dalloc(h, &pdv, (size_t)d.nzh * d.PH * nr);
    if (ce == cudaSuccess) ce = dalloc(h, &icyl, (size_t)d.P);
    if (ce == cudaSuccess) ce = dalloc(h, &h->st, 1);
    if (ce == cudaSuccess) ce = dalloc(h, &h->stage, (size_t)nrr * (d.nz + 2) * (d.nt + 2));
    if (ce == cudaSuccess) ce = cudaMemset(icyl, 1, (size_t)d.P);
    if (ce != cudaSuccess) { int r = cuda_fail(nullptr, ce, "device allocation"); tc_destroy(h); return r; }

    std::memset(&h->fd, 0, sizeof h->fd);
    std::memset(&h->ff, 0, sizeof h->ff);
    if (h->mixed) ce = alloc_fields(h, h->ff);
    else ce = alloc_fields(h, h->fd);
    if (ce != cudaSuccess) { int r = cuda_fail(nullptr, ce, "device allocation"); tc_destroy(h); return r; }
    h->fd.pf_l = pl; h->fd.pf_dinv = pdv; h->fd.icyl = icyl; h->fd.st = h->st;
    h->ff.pf_l = pl; h->ff.pf_dinv = pdv; h->ff.icyl = icyl; h->ff.st = h->st;

    // FFT plans and twiddles
    FFTPlan pth, pz;
    if (!make_plan(d.M, pth, h->mixed) || !make_plan(d.nz, pz, h->mixed)) {
        int r = fail(nullptr, 2003, "FFT length has a prime factor above 13"); tc_destroy(h); return r;
    }
    if (zfft_smem_bytes(d.nz, h->mixed) > 200 * 1024) {
        int r = fail(nullptr, 2003, "NZM too large for one z-FFT tile in shared memory"); tc_destroy(h); return r;
    }
    h->pd.th = pth; h->pd.z = pz; h->pf.th = pth; h->pf.z = pz;
    ce = h->mixed ? upload_plans(h, h->pf) : upload_plans(h, h->pd);
    if (ce != cudaSuccess) { int r = cuda_fail(nullptr, ce, "twiddle upload"); tc_destroy(h); return r; }

    ce = cudaMallocHost((void**)&h->st_host, sizeof(StepState));
    if (ce != cudaSuccess) { int r = cuda_fail(nullptr, ce, "pinned allocation"); tc_destroy(h); return r; }
    std::memset(h->st_host, 0, sizeof(StepState));
    h->st_host->dt_factored = std::numeric_limits<double>::quiet_NaN();   // no factors yet
    ce = cudaMemcpy(h->st, h->st_host, sizeof(StepState), cudaMemcpyHostToDevice);
    if (ce != cudaSuccess) { int r = cuda_fail(nullptr, ce, "state upload"); tc_destroy(h); return r; }

    launch_pressure_factors(h->stream, d, h->c, pl, pdv);
    h->ff.ptri_ff = h->ptri_ff;
    h->ff.tma = nullptr;
    h->fd.tma = nullptr;
    h->maps_ok = make_march_maps(h);   // built, but the cached march is the default (tc_use_tma)
    if (h->ptri_ff) {
        float2* pu = nullptr;
        ce = dalloc(h, &pu, (size_t)nr);
        if (ce != cudaSuccess) { int r = cuda_fail(nullptr, ce, "device allocation"); tc_destroy(h); return r; }
        launch_pressure_factors_ff(h->stream, d, h->c, pl, pdv, pu);
        h->ff.pl_ff = reinterpret_cast<const float2*>(pl);
        h->ff.pdi_ff = reinterpret_cast<const float2*>(pdv);
        h->ff.pu_ff = pu;
    }
    ce = cudaStreamSynchronize(h->stream);
    if (ce != cudaSuccess) { int r = cuda_fail(nullptr, ce, "pressure factors"); tc_destroy(h); return r; }
    *out = h;
    return 0;
}

int tc_create(const tc_bou* cfg, tc_handle** out) { return tc_create_ex(cfg, TC_PREC_FP64, out); }

int tc_get_bou(const tc_handle* h, tc_bou* out) {
    if (!h || !out) return 2000;
    *out = h->bou;
    return 0;
}

int tc_use_tma(tc_handle* h, int enable) {
    if (int r = check(h)) return r;
    if (enable && !h->maps_ok) return fail(h, 2019, "no TMA descriptors for this handle (FP64, or nthm not a "
                                                   "multiple of 4 or below 64)");
    h->ff.tma = enable ? &h->maps : nullptr;
    return 0;
}

int tc_precision(const tc_handle* h) {
    return h ? (h->ptri_ff ? TC_PREC_MIXED_FF : h->mixed ? TC_PREC_MIXED : TC_PREC_FP64) : -1;
}

void tc_destroy(tc_handle* h) {
    if (!h) return;
    if (h->stream) cudaStreamSynchronize(h->stream);
    else cudaDeviceSynchronize();
    for (void* p : h->allocs) cudaFree(p);
    for (cudaEvent_t e : h->pool) cudaEventDestroy(e);
    if (h->st_host) cudaFreeHost(h->st_host);
    delete h;
}

// ---- host buffers for state transfers -------------------------------------
//
// Page-locked host memory on transparent huge pages.  On the GB300 host
// (64 KiB base pages, 512 MiB huge pages) a 13 GB state copy from or into
// cudaHostAlloc'd memory ran at 190 GB/s right after allocation but slowed
// to 25-60 GB/s once the GPU had run kernels for seconds in between
// (tc_set_state of the 1024x768x512 state: 145, 531, 725 ms in three
// rounds of 20 steps), while the same copies from anonymous memory on huge
// pages registered with cudaHostRegister stayed at 68 ms in every round.

namespace {
std::mutex g_host_mu;
std::map<void*, std::pair<void*, size_t>> g_host;   // buffer -> (mapping, length)

size_t huge_page_bytes() {
    size_t hp = 0;
    if (FILE* f = std::fopen("/sys/kernel/mm/transparent_hugepage/hpage_pmd_size", "r")) {
        unsigned long long v = 0;
        if (std::fscanf(f, "%llu", &v) == 1) hp = (size_t)v;
        std::fclose(f);
    }
    return hp >= 4096 && hp <= (size_t(1) << 30) ? hp : (size_t(2) << 20);
}
}  // namespace

int tc_host_alloc(size_t bytes, void** ptr) {
    if (!ptr || bytes == 0) return fail(nullptr, 2000, "tc_host_alloc: null pointer or zero size");
    *ptr = nullptr;
    const size_t hp = huge_page_bytes();
    const size_t span = (bytes + hp - 1) / hp * hp;
    const size_t len = span + hp;                                      // room to align the start
    void* base = mmap(nullptr, len, PROT_READ | PROT_WRITE, MAP_PRIVATE | MAP_ANONYMOUS, -1, 0);
    if (base == MAP_FAILED) return fail(nullptr, 1002, "tc_host_alloc: mmap failed");
    void* p = (void*)(((uintptr_t)base + hp - 1) / hp * hp);
    madvise(p, span, MADV_HUGEPAGE);          // advisory: without huge pages the buffer still works
    std::memset(p, 0, bytes);                 // fault the pages in before they are locked
    cudaError_t e = cudaHostRegister(p, bytes, cudaHostRegisterDefault);
    if (e != cudaSuccess) {
        munmap(base, len);
        return cuda_fail(nullptr, e, "tc_host_alloc: cudaHostRegister");
    }
    std::lock_guard<std::mutex> lk(g_host_mu);
    g_host[p] = {base, len};
    *ptr = p;
    return 0;
}

int tc_host_free(void* ptr) {
    std::pair<void*, size_t> m;
    {
        std::lock_guard<std::mutex> lk(g_host_mu);
        auto it = g_host.find(ptr);
        if (it == g_host.end()) return fail(nullptr, 2000, "tc_host_free: not a tc_host_alloc buffer");
        m = it->second;
        g_host.erase(it);
    }
    cudaError_t e = cudaHostUnregister(ptr);
    munmap(m.first, m.second);
    return e == cudaSuccess ? 0 : cuda_fail(nullptr, e, "tc_host_free: cudaHostUnregister");
}

int tc_set_tmax(tc_handle* h, double tmax) {
    if (int r = check(h)) return r;
    h->bou.tmax = tmax;
    h->k.tmax = tmax;
    return 0;
}

int tc_set_stream(tc_handle* h, void* s) {
    if (int r = check(h)) return r;
    h->stream = (cudaStream_t)s;
    return 0;
}

// ---- state transfer --------------------------------------------------------

// Host array (reference layout) -> device field: one copy into the staging
// buffer (by the copy engine; from pinned host memory it runs at the
// CPU-GPU link rate, about 200 GB/s on GB300, faster and steadier than
// transpose kernels that read or write host memory themselves, measured
// 150-180 GB/s and down to 30 GB/s), then the layout transpose on the device.
template <typename T>
static int upload(tc_handle* h, const double* src, T* dst, int nk, int halo) {
    const Dims& d = h->d;
    size_t n = (size_t)(d.nr + 1) * (d.nz + 2 * halo) * (d.nt + 2 * halo);
    CK(cudaMemcpyAsync(h->stage, src, n * sizeof(double), cudaMemcpyHostToDevice, h->stream), "H2D copy");
    L(h, K_LAYOUT, 1, [&] { launch_to_device(h->stream, d, (const double*)h->stage, dst, nk, halo); });
    return 0;
}

// Device field -> host array.  Asynchronous: the caller synchronises the
// stream once after its last download (stream order keeps the staging
// buffer's copies apart).
template <typename T>
static int download(tc_handle* h, const T* src, double* dst, int nk, int halo) {
    const Dims& d = h->d;
    size_t n = (size_t)(d.nr + 1) * (d.nz + 2 * halo) * (d.nt + 2 * halo);
    L(h, K_LAYOUT, 1, [&] { launch_to_host(h->stream, d, src, h->stage, nk, halo); });
    CK(cudaMemcpyAsync(dst, h->stage, n * sizeof(double), cudaMemcpyDeviceToHost, h->stream), "D2H copy");
    return 0;
}

// The mixed path keeps an FP32 copy of the FP64 pressure for the momentum rhs.
static void refresh_prf(tc_handle*, FieldsT<double>&) {}
static void refresh_prf(tc_handle* h, FieldsT<float>& f) {
    const long long n = (long long)h->d.P * h->d.nr;
    L(h, K_LAYOUT, 1, [&] { launch_round_to_float(h->stream, f.pr, f.prf, n); });
}

template <typename T>
static int set_state_t(tc_handle* h, const double* qt, const double* qr, const double* qz, const double* pr) {
    const Dims& d = h->d;
    FieldsT<T>& f = F<T>(h);
    const size_t cells = (size_t)d.P * d.nr, faces = (size_t)d.P * (d.nr + 1);
    if (int r = upload(h, qt, f.qt, d.nr, 1)) return r;
    if (int r = upload(h, qr, f.qr, d.nr + 1, 1)) return r;
    if (int r = upload(h, qz, f.qz, d.nr, 1)) return r;
    if (pr) { if (int r = upload(h, pr, f.pr, d.nr, 1)) return r; }
    else CK(cudaMemsetAsync(f.pr, 0, cells * sizeof(double), h->stream), "memset");
    CK(cudaMemsetAsync(f.ru1, 0, cells * sizeof(T), h->stream), "memset");
    CK(cudaMemsetAsync(f.ru2, 0, faces * sizeof(T), h->stream), "memset");
    CK(cudaMemsetAsync(f.ru3, 0, cells * sizeof(T), h->stream), "memset");
    refresh_prf(h, f);
    CK(cudaStreamSynchronize(h->stream), "set_state sync");
    return 0;
}

int tc_set_state(tc_handle* h, const double* qt, const double* qr, const double* qz, const double* pr) {
    if (int r = check(h)) return r;
    if (!qt || !qr || !qz) return fail(h, 2000, "null field");
    return h->mixed ? set_state_t<float>(h, qt, qr, qz, pr) : set_state_t<double>(h, qt, qr, qz, pr);
}

template <typename T>
static int get_state_t(tc_handle* h, double* qt, double* qr, double* qz, double* pr) {
    const Dims& d = h->d;
    FieldsT<T>& f = F<T>(h);
    if (qt) if (int r = download(h, (const T*)f.qt, qt, d.nr, 1)) return r;
    if (qr) if (int r = download(h, (const T*)f.qr, qr, d.nr + 1, 1)) return r;
    if (qz) if (int r = download(h, (const T*)f.qz, qz, d.nr, 1)) return r;
    if (pr) if (int r = download(h, (const double*)f.pr, pr, d.nr, 1)) return r;
    CK(cudaStreamSynchronize(h->stream), "get_state sync");
    return 0;
}

int tc_get_state(tc_handle* h, double* qt, double* qr, double* qz, double* pr) {
    if (int r = check(h)) return r;
    return h->mixed ? get_state_t<float>(h, qt, qr, qz, pr) : get_state_t<double>(h, qt, qr, qz, pr);
}

template <typename T>
static int field_io(tc_handle* h, int which, double* out, const double* in) {
    const Dims& d = h->d;
    FieldsT<T>& f = F<T>(h);
    int halo = which <= TC_F_DPH ? 1 : 0, nk = d.nr;
    T* p = nullptr;
    double* pp = nullptr;
    switch (which) {
        case TC_F_QT: p = f.qt; break;
        case TC_F_QR: p = f.qr; nk = d.nr + 1; break;
        case TC_F_QZ: p = f.qz; break;
        case TC_F_PR: pp = f.pr; break;
        case TC_F_DPH: p = f.phi; break;
        case TC_F_RHS_T: p = f.rhs_t; break;
        case TC_F_RHS_R: p = f.rhs_r; nk = d.nr + 1; break;
        case TC_F_RHS_Z: p = f.rhs_z; break;
        case TC_F_RU1: p = f.ru1; break;
        case TC_F_RU2: p = f.ru2; nk = d.nr + 1; break;
        case TC_F_RU3: p = f.ru3; break;
        case TC_F_DQ: p = f.h_t; break;
        case TC_F_HR: p = f.h_r; nk = d.nr + 1; break;
        case TC_F_QCAP: p = f.h_z; break;
        default: return fail(h, 2004, "unknown field id");
    }
    if (!p && !pp) return fail(h, 2005, "field not allocated (call tc_explicit_terms first)");
    if (out) {
        int r = pp ? download(h, (const double*)pp, out, nk, halo) : download(h, (const T*)p, out, nk, halo);
        if (r) return r;
        CK(cudaStreamSynchronize(h->stream), "get_field sync");
        return 0;
    }
    int r = pp ? upload(h, in, pp, nk, halo) : upload(h, in, p, nk, halo);
    if (r) return r;
    if (pp) refresh_prf(h, f);
    CK(cudaStreamSynchronize(h->stream), "set_field sync");
    return 0;
}

int tc_get_field(tc_handle* h, int which, double* out) {
    if (int r = check(h)) return r;
    if (!out) return fail(h, 2000, "null output");
    return h->mixed ? field_io<float>(h, which, out, nullptr) : field_io<double>(h, which, out, nullptr);
}

int tc_set_field(tc_handle* h, int which, const double* in) {
    if (int r = check(h)) return r;
    if (!in) return fail(h, 2000, "null input");
    return h->mixed ? field_io<float>(h, which, nullptr, in) : field_io<double>(h, which, nullptr, in);
}

// ---- the step ----------------------------------------------------------------

template <typename T>
static void enqueue_substeps(tc_handle* h) {
    cudaStream_t s = h->stream;
    const FieldsT<T>& f = F<T>(h);
    const CoefT<T>& cv = CF<T>(h);
    const PlansT<T>& p = PL<T>(h);
    for (int sub = 0; sub < h->k.nsst; ++sub) {
        L(h, K_MOMENTUM, 1, [&] { launch_momentum(s, MODE_FUSED, h->d, cv, h->k, f, sub); });
        L(h, K_RADIAL, 1, [&] { launch_radial_solve(s, h->d, f, sub); });
        L(h, K_DIVFFT, 1, [&] { launch_div_fft(s, h->d, cv, h->k, f, p, sub, false); });
        L(h, K_ZFFT, 1, [&] { launch_zfft(s, h->d, f, p, false); });
        L(h, K_PTRI, 1, [&] { launch_pressure_tridiag(s, h->d, h->c, f); });
        L(h, K_ZFFT, 1, [&] { launch_zfft(s, h->d, f, p, true); });
        L(h, K_THINV, 1, [&] { launch_theta_inverse(s, h->d, f, p); });
        L(h, K_CORRECT, 1, [&] { launch_correct(s, h->d, h->c, CF<T>(h), h->k, f, sub, true, true); });
    }
}

template <typename T>
static void enqueue_begin(tc_handle* h, int mode, double dt, double time) {
    L(h, K_CONTROL, 1, [&] { launch_begin_step(h->stream, h->k, h->st, mode, dt, time); });
    if (h->k.patterned) L(h, K_CONTROL, 1, [&] { launch_slip(h->stream, h->d, h->k, F<T>(h)); });
    L(h, K_CONTROL, 1, [&] { launch_factors(h->stream, h->d, h->c, h->k, F<T>(h)); });
}

int tc_time_marcher(tc_handle* h, double dt, double time) {
    if (int r = check(h)) return r;
    if (h->mixed) { enqueue_begin<float>(h, 0, dt, time); enqueue_substeps<float>(h); }
    else { enqueue_begin<double>(h, 0, dt, time); enqueue_substeps<double>(h); }
    CK(cudaGetLastError(), "tc_time_marcher launch");
    return 0;
}

int tc_kernels_per_step(const tc_handle* h) {
    if (!h) return 0;
    return 2 + (h->k.patterned ? 1 : 0) + 8 * h->k.nsst;
}

long long tc_device_bytes(const tc_handle* h) { return h ? h->bytes : 0; }

namespace {
__global__ void set_clock_kernel(StepState* st, int ntime, double time) {
    st->ntime = ntime;
    st->time = time;
    st->halt = 0;
    st->errorcode = 0;
}
}  // namespace

static int read_state(tc_handle* h) {
    CK(cudaMemcpyAsync(h->st_host, h->st, sizeof(StepState), cudaMemcpyDeviceToHost, h->stream), "state read");
    CK(cudaStreamSynchronize(h->stream), "state sync");
    return 0;
}

template <typename T>
static void enqueue_run(tc_handle* h, int nsteps, int nt0, double t0) {
    cudaStream_t s = h->stream;
    const FieldsT<T>& f = F<T>(h);
    L(h, K_CONTROL, 1, [&] { set_clock_kernel<<<1, 1, 0, s>>>(h->st, nt0, t0); });
    for (int n = 0; n < nsteps; ++n) {
        L(h, K_REDUCE, 2, [&] { launch_cfl(s, h->d, h->c, CF<T>(h), h->k, f); });
        enqueue_begin<T>(h, 1, 0.0, 0.0);
        enqueue_substeps<T>(h);
        L(h, K_CONTROL, 1, [&] { launch_end_step(s, h->k, h->st); });
        L(h, K_REDUCE, 4, [&] {
            launch_velocity_stats(s, h->d, h->c, h->k, f, true);
            launch_check_divergence(s, h->d, h->c, CF<T>(h), h->k, f, true);
        });
        L(h, K_CONTROL, 1, [&] { launch_finish_step(s, h->k, h->st); });
    }
}

int tc_run(tc_handle* h, int nsteps, int* ntime, double* time, double* dt) {
    if (int r = check(h)) return r;
    if (!ntime || !time || !dt) return fail(h, 2000, "null argument");
    if (h->mixed) enqueue_run<float>(h, nsteps, *ntime, *time);
    else enqueue_run<double>(h, nsteps, *ntime, *time);
    CK(cudaGetLastError(), "tc_run launch");
    if (int r = read_state(h)) return r;
    *ntime = h->st_host->ntime;
    *time = h->st_host->time;
    *dt = h->st_host->dt;
    return h->st_host->halt ? h->st_host->errorcode : 0;
}

// ---- per-routine entry points ---------------------------------------------

int tc_begin_step(tc_handle* h, double dt, double time) {
    if (int r = check(h)) return r;
    if (h->mixed) enqueue_begin<float>(h, 0, dt, time);
    else enqueue_begin<double>(h, 0, dt, time);
    h->sub = 0;
    return 0;
}

int tc_set_substep(tc_handle* h, int ns) {
    if (int r = check(h)) return r;
    if (ns < 1 || ns > h->k.nsst) return fail(h, 2006, "substep out of range");
    h->sub = ns - 1;
    return 0;
}

template <typename T>
static int ensure_h(tc_handle* h) {
    const Dims& d = h->d;
    FieldsT<T>& f = F<T>(h);
    cudaError_t ce = cudaSuccess;
    if (!f.h_t) ce = dalloc(h, &f.h_t, (size_t)d.P * d.nr);
    if (ce == cudaSuccess && !f.h_r) ce = dalloc(h, &f.h_r, (size_t)d.P * (d.nr + 1));
    if (ce == cudaSuccess && !f.h_z) ce = dalloc(h, &f.h_z, (size_t)d.P * d.nr);
    if (ce != cudaSuccess) return cuda_fail(h, ce, "explicit-term arrays");
    return 0;
}

// comp: -1 all three components, else 0 (qt), 1 (qr) or 2 (qz) alone.
template <typename T>
static int routine(tc_handle* h, int which, int comp) {
    cudaStream_t s = h->stream;
    const int mask = comp < 0 ? 7 : (1 << comp);
    const int comp0 = comp < 0 ? 0 : comp, ncomp = comp < 0 ? 3 : 1;
    if (which <= 1) {
        if (int r = ensure_h<T>(h)) return r;
    }
    const FieldsT<T>& f = F<T>(h);
    const CoefT<T>& cv = CF<T>(h);
    const PlansT<T>& p = PL<T>(h);
    const int sub = h->sub;
    switch (which) {
        case 0:  // ExplicitTermsQT/QR/QZ
            L(h, K_MOMENTUM, 1, [&] { launch_momentum(s, MODE_EXPLICIT, h->d, cv, h->k, f, sub, mask); });
            break;
        case 1:  // ImplicitAndUpdateQ* with SolveImpEqnUpdate_Q*
            L(h, K_MOMENTUM, 1, [&] { launch_momentum(s, MODE_IMPLICIT, h->d, cv, h->k, f, sub, mask); });
            L(h, K_RADIAL, 1, [&] { launch_radial_solve(s, h->d, f, sub, comp0, ncomp); });
            break;
        case 2:
            L(h, K_MOMENTUM, 1, [&] { launch_momentum(s, MODE_FUSED, h->d, cv, h->k, f, sub); });
            break;
        case 3:
            L(h, K_RADIAL, 1, [&] { launch_radial_solve(s, h->d, f, sub, comp0, ncomp); });
            break;
        case 4:
            L(h, K_DIVFFT, 1, [&] { launch_divergence(s, h->d, cv, h->k, f, sub); });
            break;
        case 5:
            L(h, K_DIVFFT, 1, [&] { launch_div_fft(s, h->d, cv, h->k, f, p, sub, true); });
            L(h, K_ZFFT, 1, [&] { launch_zfft(s, h->d, f, p, false); });
            L(h, K_PTRI, 1, [&] { launch_pressure_tridiag(s, h->d, h->c, f); });
            L(h, K_ZFFT, 1, [&] { launch_zfft(s, h->d, f, p, true); });
            L(h, K_THINV, 1, [&] { launch_theta_inverse(s, h->d, f, p); });
            break;
        case 6:
            L(h, K_CORRECT, 1, [&] { launch_correct(s, h->d, h->c, CF<T>(h), h->k, f, sub, true, false); });
            break;
        default:
            L(h, K_CORRECT, 1, [&] { launch_correct(s, h->d, h->c, CF<T>(h), h->k, f, sub, false, true); });
            break;
    }
    return 0;
}

static int run_routine(tc_handle* h, int which, int comp = -1) {
    if (int r = check(h)) return r;
    return h->mixed ? routine<float>(h, which, comp) : routine<double>(h, which, comp);
}

int tc_explicit_terms(tc_handle* h) { return run_routine(h, 0); }
int tc_implicit_and_update(tc_handle* h) { return run_routine(h, 1); }
int tc_explicit_and_rhs(tc_handle* h) { return run_routine(h, 2); }
int tc_solve_imp_eqn_update(tc_handle* h) { return run_routine(h, 3); }
int tc_explicit_terms_qt(tc_handle* h) { return run_routine(h, 0, 0); }
int tc_explicit_terms_qr(tc_handle* h) { return run_routine(h, 0, 1); }
int tc_explicit_terms_qz(tc_handle* h) { return run_routine(h, 0, 2); }
int tc_implicit_and_update_qt(tc_handle* h) { return run_routine(h, 1, 0); }
int tc_implicit_and_update_qr(tc_handle* h) { return run_routine(h, 1, 1); }
int tc_implicit_and_update_qz(tc_handle* h) { return run_routine(h, 1, 2); }
int tc_solve_imp_eqn_update_qt(tc_handle* h) { return run_routine(h, 3, 0); }
int tc_solve_imp_eqn_update_qr(tc_handle* h) { return run_routine(h, 3, 1); }
int tc_solve_imp_eqn_update_qz(tc_handle* h) { return run_routine(h, 3, 2); }
int tc_calc_local_divergence(tc_handle* h) { return run_routine(h, 4); }
int tc_solve_pressure_correction(tc_handle* h) { return run_routine(h, 5); }
int tc_correct_velocity(tc_handle* h) { return run_routine(h, 6); }
int tc_correct_pressure(tc_handle* h) { return run_routine(h, 7); }

// ---- reductions ---------------------------------------------------------------

template <typename T>
static void enqueue_reduce(tc_handle* h, int which) {
    cudaStream_t s = h->stream;
    const FieldsT<T>& f = F<T>(h);
    switch (which) {
        case 0: L(h, K_REDUCE, 2, [&] { launch_cfl(s, h->d, h->c, CF<T>(h), h->k, f); }); break;
        case 1: L(h, K_REDUCE, 2, [&] { launch_check_divergence(s, h->d, h->c, CF<T>(h), h->k, f, false); }); break;
        case 2: L(h, K_REDUCE, 2, [&] { launch_torque(s, h->d, h->c, h->k, f); }); break;
        default: L(h, K_REDUCE, 2, [&] { launch_velocity_stats(s, h->d, h->c, h->k, f, false); }); break;
    }
}

static int reduce(tc_handle* h, int which) {
    if (int r = check(h)) return r;
    if (h->mixed) enqueue_reduce<float>(h, which);
    else enqueue_reduce<double>(h, which);
    return read_state(h);
}

int tc_calc_max_cfl(tc_handle* h, double* cflm) {
    if (int r = reduce(h, 0)) return r;
    if (cflm) *cflm = h->st_host->instcfl;
    return 0;
}

int tc_check_divergence(tc_handle* h, double* qmax) {
    if (int r = reduce(h, 1)) return r;
    const double v = h->st_host->dmax;
    if (qmax) *qmax = v;
    if (v != v) return fail(h, 169, "tc_check_divergence: the velocity field holds a NaN");
    return 0;
}

int tc_calc_torque(tc_handle* h, double* inner, double* outer) {
    if (int r = reduce(h, 2)) return r;
    if (inner) *inner = h->st_host->torque[0];
    if (outer) *outer = h->st_host->torque[1];
    return 0;
}

int tc_calc_velocity_stats(tc_handle* h, double* vmax3, double* rms3) {
    if (int r = reduce(h, 3)) return r;
    for (int q = 0; q < 3; ++q) {
        if (vmax3) vmax3[q] = h->st_host->vmax[q];
        if (rms3) rms3[q] = h->st_host->rms[q];
    }
    return 0;
}

// ---- measurement helpers ---------------------------------------------------

long long tc_launch_count(const tc_handle* h) { return h ? h->launches : 0; }

int tc_kernels_per_run_step(const tc_handle* h) {
    if (!h) return 0;
    return tc_kernels_per_step(h) + 2 + 1 + 4 + 1;
}

int tc_profile(tc_handle* h, int enable) {
    if (int r = check(h)) return r;
    CK(cudaStreamSynchronize(h->stream), "profile sync");
    h->profiling = enable != 0;
    h->recs.clear();
    h->pool_used = 0;
    for (int c = 0; c < 16; ++c) { h->prof_ms[c] = 0.0; h->prof_n[c] = 0; }
    return 0;
}

int tc_profile_read(tc_handle* h, double* ms, long long* launches, int cap) {
    if (int r = check(h)) return r;
    CK(cudaStreamSynchronize(h->stream), "profile sync");
    for (const auto& r : h->recs) {
        float t = 0.f;
        CK(cudaEventElapsedTime(&t, r.a, r.b), "event time");
        h->prof_ms[r.cls] += t;
    }
    h->recs.clear();
    h->pool_used = 0;
    for (int c = 0; c < K_COUNT && c < cap; ++c) {
        if (ms) ms[c] = h->prof_ms[c];
        if (launches) launches[c] = h->prof_n[c];
    }
    return K_COUNT;
}

int tc_measure_fp64_peak(tc_handle* h, double* tflops) {
    if (int r = check(h)) return r;
    double v = measure_fp64_peak(h->stream);
    if (v < 0) return fail(h, 1002, "probe allocation failed");
    if (tflops) *tflops = v;
    return 0;
}

const char* tc_profile_name(int cls) { return (cls >= 0 && cls < K_COUNT) ? kClassNames[cls] : ""; }
