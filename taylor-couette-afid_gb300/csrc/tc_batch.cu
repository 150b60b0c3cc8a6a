// tc_batch.cu -- ensembles: many independent, unevenly sized instances
// advanced together (include/tc_capi.h, tc_ensemble_*).
//
// Each member is an ordinary handle (tc_create_ex); its device state, grid
// and coefficients are reused as they are.  One step of the ensemble is a
// fixed sequence of grouped launches, each covering every active member: the
// launch's blocks form a flat work list of (member, tile) items, a block
// reads its member from an owner table (the member of every item), its first
// item from a prefix table of item counts, and then runs the same device
// body as the single-instance kernel (tc_bodies.cuh), so
// a member's arithmetic is identical alone and in the mix.  Per step:
//   begin (dt, beta, inner-wall forcing per member), factors (one block per
//   member), then per RK substep: momentum, radial solve, divergence + theta
//   FFT, z FFT, pressure tridiagonal, inverse z FFT, inverse theta FFT,
//   correction; then end (time += dt).
// The whole step is captured once in a CUDA graph and replayed; it is
// re-captured only when members join or leave.  Members run with a fixed dt
// (from their initial CFL) or recompute dt from their CFL every step.
//
// The persistent schedule (tc_persist.cu, tc_ensemble_schedule) replaces the
// grouped launches by one cooperative launch per RK substep over the same
// work lists and device bodies, with grid-wide barriers between the phases.
//
// The schedule and the tile shapes (threads per cell tile, rows per
// theta-FFT block) are tuning knobs, chosen per ensemble by the project's
// autotuner (taylor-couette-afid_gb300/autotune.py) through
// tc_ensemble_schedule and tc_ensemble_tune.

#include <algorithm>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "tc_ens.cuh"
#include "tc_handle.h"

namespace tcgb {
namespace ens {

// ---- per-step control ----------------------------------------------------

// Fixed-dt members: TimeMarcher with the member's dt (mode 0).  Variable-dt
// members: main.F90:156-174 from the CFL number the CFL kernel just reduced
// (mode 1), which may raise 165/166.
template <typename T>
__global__ void ens_begin_kernel(const InstT<T>* inst, int n) {
    int m = blockIdx.x * blockDim.x + threadIdx.x;
    if (m >= n) return;
    StepState* st = inst[m].f.st;
    if (st->halt) return;
    begin_step_body(inst[m].k, st, inst[m].vdt, st->dt, st->time);
}

// time = time + dt; a variable-dt member that raised an error stops here,
// as the reference's run would (main.F90:229-259).
template <typename T>
__global__ void ens_end_kernel(const InstT<T>* inst, int n) {
    int m = blockIdx.x * blockDim.x + threadIdx.x;
    if (m >= n) return;
    StepState* st = inst[m].f.st;
    if (st->halt) return;
    st->time = st->time + st->dt;
    st->ntime += 1;
    if (st->errorcode != 0) st->halt = 1;
    st->instcfl = kCflFloor;
}

template <typename T>
__global__ void ens_factors_kernel(const InstT<T>* inst) {
    const InstT<T>& I = inst[blockIdx.x];
    if (I.f.st->halt) return;
    factors_body(I.d, I.c, I.k, I.f.st, I.f.Fd, I.f.corrd, I.f.scal, I.f.F, I.f.corr);
}

__global__ void ens_init_kernel(StepState* st, double dt, double time, int ntime) {
    st->dt = dt;
    st->time = time;
    st->ntime = ntime;
    st->halt = 0;
    st->errorcode = 0;
    st->instcfl = kCflFloor;
    st->dt_factored = __longlong_as_double(0x7ff8000000000000LL);   // NaN: factor on the first step
}

// CalcMaxCFL of the variable-dt members: item = (k, kCflTiles consecutive
// tiles of blockDim.x cells); block maximum, then an atomic maximum on the
// bits of the member's instcfl (the order of non-negative doubles is the
// order of their bit patterns).  A block reduces up to kCflTiles tiles
// before its one atomic: with one tile an item the atomics on the few
// members' instcfl were the bottleneck of the phase.
constexpr int kCflTiles = 8;

template <typename T>
__global__ void __launch_bounds__(256) ens_cfl_kernel(const InstT<T>* inst, const int* prefix, const int* owner) {
    __shared__ double sh[32];
    const long long item = blockIdx.x;
    const int m = __ldg(owner + item);
    const InstT<T>& I = inst[m];
    if (I.f.st->halt) return;
    const long long local = item - prefix[m];
    const int tiles = (int)((I.d.P + blockDim.x - 1) / blockDim.x);
    const int chunks = (tiles + kCflTiles - 1) / kCflTiles;
    const int k = (int)((unsigned)local / (unsigned)chunks);
    const int ch = (int)(local - (long long)k * chunks);
    const int t1 = min(tiles, (ch + 1) * kCflTiles);
    double v = 0.0;
    for (int tt = ch * kCflTiles; tt < t1; ++tt) {
        const long long flat = (long long)tt * blockDim.x + threadIdx.x;
        if (flat < I.d.P) {
            const int j = (int)((unsigned)flat / (unsigned)I.d.nt), i = (int)flat - j * I.d.nt;
            v = fmax(v, cfl_cell(I.d, I.c, I.cv, I.k.dxt, I.k.dxz, I.f, i, j, k));
        }
    }
    for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, o));
    const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
    if (l == 0) sh[w] = v;
    __syncthreads();
    if (w == 0) {
        v = (l < (int)(blockDim.x >> 5)) ? sh[l] : 0.0;
        for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, o));
        if (l == 0)
            atomicMax(reinterpret_cast<unsigned long long*>(&I.f.st->instcfl), (unsigned long long)__double_as_longlong(v));
    }
}

// ---- grouped substep phases ---------------------------------------------------

// Register targets of the heavier grouped kernels, as minimum resident
// blocks of 256 threads (smaller tiles fit proportionally more): 4 blocks =
// 64 registers, 3 = 80, 2 = 128.  As for the single-run kernels, more
// resident warps beat the few values a thread would otherwise keep in
// flight; the radial sweeps (FP64; FP32 two columns a thread) keep 80
// and the two-cell momentum bodies (FP64 and packed FP32) 128.
template <typename T> struct EnsBlocks { static constexpr int momentum = 2, radial = 3, ptri = 4; };
template <> struct EnsBlocks<float> { static constexpr int momentum = 2, radial = 3, ptri = 4; };

// momentum: item = (chunk of kMomChunk radial levels, tile of TPB pairs of
// theta-neighbouring columns), each thread marching its two columns in r in
// packed FP32 (momentum_column_x2); for FP64 (no marching) a chunk is one
// level and a thread a pair of cells (momentum_pair)
template <typename T>
__global__ void __launch_bounds__(256, EnsBlocks<T>::momentum) ens_momentum_kernel(const InstT<T>* inst, const int* prefix, const int* owner, int sub) {
    const long long item = blockIdx.x;
    const int m = __ldg(owner + item);
    const InstT<T>& I = inst[m];
    if (I.f.st->halt) return;
    const long long local = item - prefix[m];
    const long long units = mom_units<T>(I.d.P);
    const int tiles = (int)((units + blockDim.x - 1) / blockDim.x);
    const int chunk = (int)((unsigned)local / (unsigned)tiles);
    const long long flat = (local - (long long)chunk * tiles) * blockDim.x + threadIdx.x;
    if constexpr (MomMarch<T>::value) {
        // The block's member and chunk are one: its arguments and the chunk's
        // per-level coefficients are copied to shared memory once, so that the
        // march reads them there instead of chasing the member's pointers in
        // global memory at every level (two dependent loads a coefficient).
        __shared__ MarchCoef ctab[kMomChunk];
        __shared__ MomArgs<float> sma;
        const int k0 = chunk * kMomChunk, k1 = min(k0 + kMomChunk, I.d.nr);
        constexpr int kWords = (int)(sizeof(MomArgs<float>) / sizeof(int));
        static_assert(sizeof(MomArgs<float>) % sizeof(int) == 0, "MomArgs copied as ints");
        for (int w = threadIdx.x; w < kWords; w += blockDim.x)
            reinterpret_cast<int*>(&sma)[w] = reinterpret_cast<const int*>(&I.ma[sub])[w];
        for (int e = threadIdx.x; e < (k1 - k0) * kMarchCoefN; e += blockDim.x)
            reinterpret_cast<float*>(ctab)[e] =
                march_coef_entry(I.cv, I.ma[sub], I.d.nr + 1, k0 + e / kMarchCoefN, e % kMarchCoefN);
        __syncthreads();
        if (flat >= units) return;
        int i, j;
        mom_unit_cell<T>((int)flat, I.d.nt, i, j);
        momentum_column_x2<true>(I.d, I.cv, sma, i, j, k0, k1, ctab);
    } else {
        if (flat >= units) return;
        int i, j;
        mom_unit_cell<T>((int)flat, I.d.nt, i, j);
        mom_unit(I.d, I.cv, I.ma[sub], i, j, chunk);
    }
}

// cell-wise phases: item = (k, tile of TPB consecutive (j, i) cells)

template <typename T>
__global__ void __launch_bounds__(256) ens_correct_kernel(const InstT<T>* inst, const int* prefix, const int* owner, int sub) {
    const long long item = blockIdx.x;
    const int m = __ldg(owner + item);
    const InstT<T>& I = inst[m];
    if (I.f.st->halt) return;
    const long long local = item - prefix[m];
    const long long units = cell_units<T>(I.d.P);
    const int tiles = (int)((units + blockDim.x - 1) / blockDim.x);
    const int k = (int)((unsigned)local / (unsigned)tiles);
    const long long flat = (local - (long long)k * tiles) * blockDim.x + threadIdx.x;
    if (flat >= units) return;
    corr_unit(I.d, I.f, sub, (int)flat, k);
}

// column-wise: item = (component, TPB consecutive (z, theta) columns)
template <typename T>
__global__ void __launch_bounds__(256, EnsBlocks<T>::radial) ens_radial_kernel(const InstT<T>* inst, const int* prefix, const int* owner, int sub) {
    const long long item = blockIdx.x;
    const int m = __ldg(owner + item);
    const InstT<T>& I = inst[m];
    if (I.f.st->halt) return;
    const long long local = item - prefix[m];
    const long long units = cell_units<T>(I.d.P);
    const int tiles = (int)((units + blockDim.x - 1) / blockDim.x);
    const int comp = (int)((unsigned)local / (unsigned)tiles);
    const long long u = (local - (long long)comp * tiles) * blockDim.x + threadIdx.x;
    if (u >= units) return;
    rad_unit(I.d, I.f, sub, u, comp);
}

// mode-wise: item = TPB consecutive (kz, kt) modes
// FF: the members' pressure solve (ptri_solve); one precision per ensemble
template <typename T, int FF>
__global__ void __launch_bounds__(256, (std::is_same<T, float>::value && FF == 0) ? 3 : EnsBlocks<T>::ptri) ens_ptri_kernel(const InstT<T>* inst, const int* prefix, const int* owner) {
    const long long item = blockIdx.x;
    const int m = __ldg(owner + item);
    const InstT<T>& I = inst[m];
    if (I.f.st->halt) return;
    const long long t = (item - prefix[m]) * blockDim.x + threadIdx.x;
    if (t >= (long long)I.d.nz * I.d.PH) return;
    ptri_solve<T, FF>(I.d, I.c, I.f, t);
}

// row-wise FFT phases: item = I.rows (I.rows_inv) consecutive (k, j) rows of
// the item's member, so that a block holds about as many points for a short
// theta line as for a long one
template <typename T>
__global__ void __launch_bounds__(128) ens_divfft_kernel(const InstT<T>* inst, const int* prefix, const int* owner, int sub) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const long long item = blockIdx.x;
    const int m = __ldg(owner + item);
    const InstT<T>& I = inst[m];
    if (I.f.st->halt) return;
    div_fft_rows_n<false, T>(I.d, I.cv, (T)I.k.dxt, (T)I.k.dxz, I.f, I.p.th, I.p.tw_th, I.p.twr, I.k.fft_norm, sub,
                             (item - prefix[m]) * I.rows, reinterpret_cast<typename V2<T>::type*>(smem_raw),
                             I.rows, I.lg_rows);
}

template <typename T>
__global__ void __launch_bounds__(128) ens_thinv_kernel(const InstT<T>* inst, const int* prefix, const int* owner) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const long long item = blockIdx.x;
    const int m = __ldg(owner + item);
    const InstT<T>& I = inst[m];
    if (I.f.st->halt) return;
    thinv_rows_n<T>(I.d, I.f, I.p.th, I.p.tw_th, I.p.twr, (item - prefix[m]) * I.rows_inv,
                    reinterpret_cast<typename V2<T>::type*>(smem_raw), I.rows_inv, I.lg_rows_inv);
}

// Rows per theta-FFT block of a member with M-point half lines: the largest
// power of two up to 32 with rows * M <= span points (the single-run kernels'
// rule: 512 for the divergence + forward FFT, 1024 for the inverse).
int rows_for(int M, int span) {
    int R = 1;
    while (R < 32 && (R * 2) * M <= span) R *= 2;
    return R;
}

// z FFT: item = (plane k, ZEns::cols consecutive kt columns)
// z-FFT block shape of the grouped kernels: columns per item and threads.
// On the 96-member C4 ensemble (FP32, 7.10 ms a step) 8 columns of 128
// threads beat 4 x 128 (7.33), 8 x 64 (7.14), 16 x 256 (7.18), 16 x 128
// (7.23), 8 x 256 (7.42) and 8 x 512 (7.89); FP64 does not depend on it.
template <typename T> struct ZEns { static constexpr int cols = 4, threads = 128; };
template <> struct ZEns<float> { static constexpr int cols = 8, threads = 128; };

template <typename T>
__global__ void __launch_bounds__(ZEns<T>::threads) ens_zfft_kernel(const InstT<T>* inst, const int* prefix, const int* owner, int inv) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const long long item = blockIdx.x;
    const int m = __ldg(owner + item);
    const InstT<T>& I = inst[m];
    if (I.f.st->halt) return;
    const int local = (int)(item - prefix[m]);
    constexpr int ZC = ZEns<T>::cols;
    const int groups = (I.d.PH + ZC - 1) / ZC;
    const int kplane = local / groups, g = local - kplane * groups;
    zfft_tile<ZC>(I.d, I.f, I.p.z, I.p.tw_z, inv, g * ZC, kplane, reinterpret_cast<typename V2<T>::type*>(smem_raw));
}

int ceil_div(long long a, long long b) { return (int)((a + b - 1) / b); }

}  // namespace ens
}  // namespace tcgb

struct tc_ensemble {
    int mixed = 0;
    int precision = TC_PREC_FP64;   // of every member (enum tc_precision_mode)
    cudaStream_t stream = nullptr;
    std::vector<tc_handle*> members;     // slot -> member (nullptr = free)
    std::vector<int> target;             // requested step count per slot (informational)
    std::vector<int> vdt;                // per slot: 1 = variable dt (CFL rule every step)
    std::vector<int> active;             // slots in the current work list
    void* inst_dev = nullptr;            // InstT<T>[active]
    int* prefix_dev = nullptr;           // PH_COUNT tables of (n+1) ints
    int* owner_dev = nullptr;            // grouped schedule: the member of every work item, phase by phase
    long long owner_off[tcgb::ens::PH_COUNT] = {0};
    int threads = 128;                   // threads per cell/column/mode tile
    int rows = 0;                        // rows per theta-FFT block (0: per member, from its line length)
    int rows_used = 0;                   // persistent schedule: rows of every member
    size_t smem_div = 0, smem_inv = 0, smem_z = 0;
    int items[tcgb::ens::PH_COUNT] = {0};
    int schedule = TC_SCHED_GROUPED;
    int persist_blocks = 0;              // resident blocks of the persistent kernel
    int persist_per_sm = 0;              // cap on its blocks per SM (0: occupancy limit)
    size_t persist_smem = 0;
    unsigned* bar = nullptr;             // persistent barrier: count, generation, error flag, spare
    double barrier_timeout = 10.0;       // seconds one persistent barrier wait may last
    bool dirty = true;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    long long launches = 0;
    int launches_per_step = 0;
    std::string err;
};

namespace tcgb {
namespace ens {

int efail(tc_ensemble* e, int code, const std::string& msg) {
    if (e) e->err = msg;
    return code;
}

int ecuda(tc_ensemble* e, cudaError_t c, const char* what) {
    return efail(e, 1000 + (int)c, std::string(what) + ": " + cudaGetErrorString(c));
}

template <typename T> FieldsT<T>& MF(tc_handle* h);
template <> FieldsT<double>& MF<double>(tc_handle* h) { return h->fd; }
template <> FieldsT<float>& MF<float>(tc_handle* h) { return h->ff; }
template <typename T> const CoefT<T>& MC(tc_handle* h);
template <> const CoefT<double>& MC<double>(tc_handle* h) { return h->c; }
template <> const CoefT<float>& MC<float>(tc_handle* h) { return h->cf; }
template <typename T> const PlansT<T>& MP(tc_handle* h);
template <> const PlansT<double>& MP<double>(tc_handle* h) { return h->pd; }
template <> const PlansT<float>& MP<float>(tc_handle* h) { return h->pf; }


template <typename T>
int rebuild(tc_ensemble* e) {
    const int n = (int)e->active.size();
    if (e->exec) { cudaGraphExecDestroy(e->exec); e->exec = nullptr; }
    if (e->graph) { cudaGraphDestroy(e->graph); e->graph = nullptr; }
    if (e->inst_dev) { cudaFree(e->inst_dev); e->inst_dev = nullptr; }
    if (e->prefix_dev) { cudaFree(e->prefix_dev); e->prefix_dev = nullptr; }
    if (e->owner_dev) { cudaFree(e->owner_dev); e->owner_dev = nullptr; }
    e->dirty = false;
    if (n == 0) return 0;
    std::vector<InstT<T>> inst(n);
    std::vector<int> prefix((size_t)PH_COUNT * (n + 1), 0);
    int maxM = 1, maxNz = 1;
    long long maxDiv = 1, maxInv = 1;    // points of the largest theta-FFT tiles
    for (int a = 0; a < n; ++a) maxM = std::max(maxM, e->members[e->active[a]]->d.M);
    const bool persistent = e->schedule == TC_SCHED_PERSISTENT;
    int R = e->rows > 0 ? e->rows : theta_rows(maxM);
    if (persistent) R = std::min(R, kPersistMaxRows);
    e->rows_used = R;
    const int TPB = persistent ? kPersistThreads : e->threads;
    for (int a = 0; a < n; ++a) {
        tc_handle* h = e->members[e->active[a]];
        InstT<T>& I = inst[a];
        I.d = h->d; I.cv = MC<T>(h); I.c = h->c; I.k = h->k; I.f = MF<T>(h); I.p = MP<T>(h);
        for (int s = 0; s < 3; ++s) I.ma[s] = make_mom_args(h->k, I.f, s);
        I.vdt = e->vdt[e->active[a]];
        const Dims& d = h->d;
        I.rows = persistent ? R : e->rows > 0 ? e->rows : rows_for(d.M, 512);
        I.rows_inv = persistent ? R : e->rows > 0 ? e->rows : rows_for(d.M, 1024);
        I.lg_rows = lines_log2(I.rows);
        I.lg_rows_inv = lines_log2(I.rows_inv);
        maxDiv = std::max(maxDiv, (long long)I.rows * d.M);
        maxInv = std::max(maxInv, (long long)I.rows_inv * d.M);
        maxNz = std::max(maxNz, d.nz);
        long long cnt[PH_COUNT];
        cnt[PH_MOM] = (long long)(MomMarch<T>::value ? ceil_div(d.nr, kMomChunk) : d.nr) *
                      ceil_div(mom_units<T>(d.P), TPB);
        cnt[PH_CORR] = (long long)d.nr * ceil_div(cell_units<T>(d.P), TPB);
        cnt[PH_RAD] = 3LL * ceil_div(cell_units<T>(d.P), TPB);
        cnt[PH_PTRI] = ceil_div((long long)d.nz * d.PH, TPB);
        cnt[PH_DIV] = ceil_div((long long)d.nr * d.nz, I.rows);
        cnt[PH_THINV] = ceil_div((long long)d.nr * d.nz, I.rows_inv);
        cnt[PH_ZFFT] = (long long)d.nr * ceil_div(d.PH, persistent ? ZCols<T>::value : ZEns<T>::cols);
        cnt[PH_FACT] = 1;
        // (level, tile of cells) for the persistent kernel; (level, kCflTiles tiles) grouped
        cnt[PH_CFL] = !I.vdt ? 0
                      : (long long)d.nr * (persistent ? ceil_div(d.P, TPB) : ceil_div(ceil_div(d.P, TPB), kCflTiles));
        for (int p = 0; p < PH_COUNT; ++p) {
            long long v = (long long)prefix[(size_t)p * (n + 1) + a] + cnt[p];
            if (v > 2000000000LL) return efail(e, 2010, "ensemble work list exceeds 2^31 items");
            prefix[(size_t)p * (n + 1) + a + 1] = (int)v;
        }
    }
    for (int p = 0; p < PH_COUNT; ++p) e->items[p] = prefix[(size_t)p * (n + 1) + n];
    typedef typename V2<T>::type C2;
    e->smem_div = (size_t)2 * maxDiv * sizeof(C2);
    e->smem_inv = (size_t)2 * maxInv * sizeof(C2);
    e->smem_z = (size_t)2 * (persistent ? ZCols<T>::value : ZEns<T>::cols) * maxNz * sizeof(C2);
    if (e->smem_div > 200 * 1024 || e->smem_inv > 200 * 1024 || e->smem_z > 200 * 1024)
        return efail(e, 2011, "ensemble FFT tile exceeds shared memory");
    cudaError_t c = cudaMalloc(&e->inst_dev, sizeof(InstT<T>) * n);
    if (c == cudaSuccess) c = cudaMalloc(&e->prefix_dev, sizeof(int) * prefix.size());
    if (c == cudaSuccess) c = cudaMemcpy(e->inst_dev, inst.data(), sizeof(InstT<T>) * n, cudaMemcpyHostToDevice);
    if (c == cudaSuccess) c = cudaMemcpy(e->prefix_dev, prefix.data(), sizeof(int) * prefix.size(), cudaMemcpyHostToDevice);
    if (c != cudaSuccess) return ecuda(e, c, "ensemble tables");
    if (persistent) {
        e->persist_smem = std::max(e->smem_div, e->smem_z);
        if (!e->bar) {
            c = cudaMalloc(&e->bar, 4 * sizeof(unsigned));
            if (c != cudaSuccess) return ecuda(e, c, "persistent barrier");
        }
        c = cudaMemset(e->bar, 0, 4 * sizeof(unsigned));
        if (c == cudaSuccess) c = prepare_persistent<T>(R, e->persist_smem, e->persist_per_sm, &e->persist_blocks);
        if (c != cudaSuccess) return ecuda(e, c, "persistent kernel setup");
        return 0;
    }
    cudaFuncSetAttribute(ens_divfft_kernel<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
    cudaFuncSetAttribute(ens_thinv_kernel<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
    cudaFuncSetAttribute(ens_zfft_kernel<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
    // A grouped block reads its member from the owner table (one load)
    // instead of searching the prefix table (about log2(n) dependent loads
    // that the streamed data evicts from L1, ahead of the member's struct,
    // its halt flag and only then its data).
    long long total = 0;
    for (int p = 0; p < PH_COUNT; ++p) { e->owner_off[p] = total; total += e->items[p]; }
    std::vector<int> owner((size_t)std::max(total, 1LL));
    for (int p = 0; p < PH_COUNT; ++p)
        for (int a = 0; a < n; ++a)
            std::fill(owner.begin() + e->owner_off[p] + prefix[(size_t)p * (n + 1) + a],
                      owner.begin() + e->owner_off[p] + prefix[(size_t)p * (n + 1) + a + 1], a);
    c = cudaMalloc(&e->owner_dev, sizeof(int) * owner.size());
    if (c == cudaSuccess) c = cudaMemcpy(e->owner_dev, owner.data(), sizeof(int) * owner.size(), cudaMemcpyHostToDevice);
    if (c != cudaSuccess) return ecuda(e, c, "ensemble owner table");
    return 0;
}

// Enqueue one step of every active member on e->stream.
template <typename T>
int enqueue_step(tc_ensemble* e) {
    const int n = (int)e->active.size();
    const InstT<T>* I = (const InstT<T>*)e->inst_dev;
    const int* pre = e->prefix_dev;
    auto P = [&](int p) { return pre + (size_t)p * (n + 1); };
    auto O = [&](int p) { return e->owner_dev + e->owner_off[p]; };
    cudaStream_t s = e->stream;
    const int nsst = e->members[e->active[0]]->k.nsst;
    if (e->schedule == TC_SCHED_PERSISTENT) {
        // one cooperative launch per substep; the first also runs CFL, begin
        // and factors, the last also end
        PersistArgs a;
        a.prefix = pre;
        a.n = n;
        for (int p = 0; p < PH_COUNT; ++p) a.items[p] = e->items[p];
        a.bar_count = e->bar;
        a.bar_gen = e->bar + 1;
        a.err = reinterpret_cast<int*>(e->bar + 2);
        a.timeout_ns = (unsigned long long)(e->barrier_timeout * 1e9);
        for (int sub = 0; sub < nsst; ++sub) {
            a.sub = sub;
            a.flags = 0;
            if (sub == 0) a.flags |= (e->items[PH_CFL] > 0 ? PF_CFL : 0) | PF_BEGIN | PF_FACT;
            if (sub == nsst - 1) a.flags |= PF_END;
            cudaError_t c = launch_persistent<T>(s, I, a, e->rows_used, e->persist_smem, e->persist_blocks);
            if (c != cudaSuccess) return ecuda(e, c, "persistent launch");
        }
        e->launches_per_step = nsst;
        return 0;
    }
    const int TPB = e->threads;
    int count = 0;
    if (e->items[PH_CFL] > 0) {
        ens_cfl_kernel<T><<<e->items[PH_CFL], TPB, 0, s>>>(I, P(PH_CFL), O(PH_CFL));
        ++count;
    }
    ens_begin_kernel<T><<<(n + 127) / 128, 128, 0, s>>>(I, n); ++count;
    ens_factors_kernel<T><<<n, 256, 0, s>>>(I); ++count;
    for (int sub = 0; sub < nsst; ++sub) {
        ens_momentum_kernel<T><<<e->items[PH_MOM], TPB, 0, s>>>(I, P(PH_MOM), O(PH_MOM), sub);
        ens_radial_kernel<T><<<e->items[PH_RAD], TPB, 0, s>>>(I, P(PH_RAD), O(PH_RAD), sub);
        ens_divfft_kernel<T><<<e->items[PH_DIV], 128, e->smem_div, s>>>(I, P(PH_DIV), O(PH_DIV), sub);
        ens_zfft_kernel<T><<<e->items[PH_ZFFT], ZEns<T>::threads, e->smem_z, s>>>(I, P(PH_ZFFT), O(PH_ZFFT), 0);
        if (e->precision == TC_PREC_MIXED_FF) ens_ptri_kernel<T, 1><<<e->items[PH_PTRI], TPB, 0, s>>>(I, P(PH_PTRI), O(PH_PTRI));
        else ens_ptri_kernel<T, 0><<<e->items[PH_PTRI], TPB, 0, s>>>(I, P(PH_PTRI), O(PH_PTRI));
        ens_zfft_kernel<T><<<e->items[PH_ZFFT], ZEns<T>::threads, e->smem_z, s>>>(I, P(PH_ZFFT), O(PH_ZFFT), 1);
        ens_thinv_kernel<T><<<e->items[PH_THINV], 128, e->smem_inv, s>>>(I, P(PH_THINV), O(PH_THINV));
        ens_correct_kernel<T><<<e->items[PH_CORR], TPB, 0, s>>>(I, P(PH_CORR), O(PH_CORR), sub);
        count += 8;
    }
    ens_end_kernel<T><<<(n + 127) / 128, 128, 0, s>>>(I, n); ++count;
    e->launches_per_step = count;
    cudaError_t c = cudaGetLastError();
    if (c != cudaSuccess) return ecuda(e, c, "ensemble launch");
    return 0;
}

template <typename T>
int capture(tc_ensemble* e) {
    cudaStream_t cap = nullptr;
    cudaError_t c = cudaStreamCreateWithFlags(&cap, cudaStreamNonBlocking);
    if (c != cudaSuccess) return ecuda(e, c, "capture stream");
    cudaStream_t saved = e->stream;
    e->stream = cap;
    c = cudaStreamBeginCapture(cap, cudaStreamCaptureModeThreadLocal);
    int r = 0;
    if (c == cudaSuccess) {
        r = enqueue_step<T>(e);
        cudaError_t c2 = cudaStreamEndCapture(cap, &e->graph);
        if (c2 != cudaSuccess && r == 0) r = ecuda(e, c2, "end capture");
    } else {
        r = ecuda(e, c, "begin capture");
    }
    e->stream = saved;
    cudaStreamDestroy(cap);
    if (r) return r;
    c = cudaGraphInstantiate(&e->exec, e->graph, 0);
    if (c != cudaSuccess) return ecuda(e, c, "graph instantiate");
    return 0;
}

// After the stream has drained: 3001 if a persistent barrier wait gave up
// since the last check (the barrier is reset for the next steps).
int check_barrier(tc_ensemble* e) {
    if (!e->bar) return 0;
    unsigned flag = 0;
    cudaError_t c = cudaMemcpy(&flag, e->bar + 2, sizeof flag, cudaMemcpyDeviceToHost);
    if (c != cudaSuccess) return ecuda(e, c, "barrier flag read");
    if (!flag) return 0;
    c = cudaMemset(e->bar, 0, 4 * sizeof(unsigned));
    if (c != cudaSuccess) return ecuda(e, c, "barrier reset");
    return efail(e, 3001, "persistent ensemble step: a grid barrier wait gave up; the steps since the last "
                          "synchronisation did not complete");
}

int prepare(tc_ensemble* e) {
    if (!e->dirty && (e->exec || e->active.empty())) return 0;
    int r = e->mixed ? rebuild<float>(e) : rebuild<double>(e);
    if (r) return r;
    if (e->active.empty()) return 0;
    return e->mixed ? capture<float>(e) : capture<double>(e);
}

}  // namespace ens
}  // namespace tcgb

using namespace tcgb;
using namespace tcgb::ens;

// The exported functions below are declared extern "C" in tc_capi.h.

int tc_ensemble_create(int precision, tc_ensemble** out) {
    if (!out) return 2000;
    if (precision != TC_PREC_FP64 && precision != TC_PREC_MIXED && precision != TC_PREC_MIXED_FF) return 2007;
    tc_ensemble* e = new tc_ensemble();
    e->mixed = precision != TC_PREC_FP64;
    e->precision = precision;
    *out = e;
    return 0;
}

void tc_ensemble_destroy(tc_ensemble* e) {
    if (!e) return;
    if (e->stream) cudaStreamSynchronize(e->stream);
    else cudaDeviceSynchronize();
    if (e->exec) cudaGraphExecDestroy(e->exec);
    if (e->graph) cudaGraphDestroy(e->graph);
    if (e->inst_dev) cudaFree(e->inst_dev);
    if (e->prefix_dev) cudaFree(e->prefix_dev);
    if (e->owner_dev) cudaFree(e->owner_dev);
    if (e->bar) cudaFree(e->bar);
    for (tc_handle* h : e->members) if (h) tc_destroy(h);
    delete e;
}

const char* tc_ensemble_last_error(const tc_ensemble* e) { return e ? e->err.c_str() : ""; }

int tc_ensemble_set_stream(tc_ensemble* e, void* stream) {
    if (!e) return 2000;
    e->stream = (cudaStream_t)stream;
    for (tc_handle* h : e->members) if (h) tc_set_stream(h, stream);
    return 0;
}

int tc_ensemble_add(tc_ensemble* e, const tc_bou* cfg, double dt, const double* qt, const double* qr,
                    const double* qz, const double* pr, int nsteps, int* slot) {
    if (!e || !cfg || !slot) return 2000;
    if (cfg->minstrt > 0 || cfg->minstrz > 0)
        return efail(e, 2012, "patterned slip (MINSTRT/MINSTRZ > 0) cannot run in an ensemble");
    for (int s : e->active)
        if (e->members[s]->k.nsst != cfg->nsst)
            return efail(e, 2012, "every member of an ensemble needs the same NSST");
    tc_handle* h = nullptr;
    int r = tc_create_ex(cfg, e->precision, &h);
    if (r) return efail(e, r, tc_last_error(nullptr));
    tc_set_stream(h, e->stream);
    r = tc_set_state(h, qt, qr, qz, pr);
    if (r) { std::string m = tc_last_error(h); tc_destroy(h); return efail(e, r, m); }
    int variable = 0;
    if (!(dt > 0.0) && cfg->idtv == 1) {
        variable = 1;                   // begin computes dt from the CFL of each step
        dt = cfg->dtmin;
    } else if (!(dt > 0.0)) {
        // main.F90:160-166 once, on the start
        double cfl = 0.0;
        r = tc_calc_max_cfl(h, &cfl);
        if (r) { std::string m = tc_last_error(h); tc_destroy(h); return efail(e, r, m); }
        dt = (cfl < 1.0e-8) ? cfg->dtmax : cfg->limitCFL / cfl;
        if (dt > cfg->dtmax) dt = cfg->dtmax;
    }
    ens_init_kernel<<<1, 1, 0, e->stream>>>(h->st, dt, 0.0, 0);
    cudaError_t c = cudaStreamSynchronize(e->stream);
    if (c != cudaSuccess) { tc_destroy(h); return ecuda(e, c, "member init"); }
    int s = -1;
    for (size_t i = 0; i < e->members.size(); ++i)
        if (!e->members[i]) { s = (int)i; break; }
    if (s < 0) {
        s = (int)e->members.size();
        e->members.push_back(nullptr);
        e->target.push_back(0);
        e->vdt.push_back(0);
    }
    e->members[s] = h;
    e->target[s] = nsteps;
    e->vdt[s] = variable;
    e->active.push_back(s);
    std::sort(e->active.begin(), e->active.end());
    e->dirty = true;
    *slot = s;
    return 0;
}

int tc_ensemble_remove(tc_ensemble* e, int slot) {
    if (!e || slot < 0 || slot >= (int)e->members.size() || !e->members[slot]) return 2000;
    if (e->stream) cudaStreamSynchronize(e->stream);
    else cudaDeviceSynchronize();
    tc_destroy(e->members[slot]);
    e->members[slot] = nullptr;
    e->active.erase(std::remove(e->active.begin(), e->active.end(), slot), e->active.end());
    e->dirty = true;
    return 0;
}

int tc_ensemble_member(tc_ensemble* e, int slot, tc_handle** h) {
    if (!e || !h || slot < 0 || slot >= (int)e->members.size() || !e->members[slot]) return 2000;
    *h = e->members[slot];
    return 0;
}

int tc_ensemble_count(const tc_ensemble* e) { return e ? (int)e->active.size() : 0; }

int tc_ensemble_target(const tc_ensemble* e, int slot) {
    if (!e || slot < 0 || slot >= (int)e->members.size() || !e->members[slot]) return -1;
    return e->target[slot];
}

int tc_ensemble_tune(tc_ensemble* e, int threads, int rows) {
    if (!e) return 2000;
    if (threads != 64 && threads != 128 && threads != 256) return efail(e, 2013, "threads must be 64, 128 or 256");
    if (rows != 0 && rows != 1 && rows != 2 && rows != 4 && rows != 8 && rows != 16 && rows != 32)
        return efail(e, 2013, "rows must be 0 (automatic) or a power of two up to 32");
    e->threads = threads;
    e->rows = rows;
    e->dirty = true;
    return 0;
}

int tc_ensemble_schedule(tc_ensemble* e, int schedule, int blocks_per_sm) {
    if (!e) return 2000;
    if (schedule != TC_SCHED_GROUPED && schedule != TC_SCHED_PERSISTENT)
        return efail(e, 2013, "schedule must be TC_SCHED_GROUPED or TC_SCHED_PERSISTENT");
    if (blocks_per_sm < 0 || blocks_per_sm > 32) return efail(e, 2013, "blocks_per_sm must be 0..32");
    if (schedule != e->schedule || blocks_per_sm != e->persist_per_sm) {
        e->schedule = schedule;
        e->persist_per_sm = blocks_per_sm;
        e->dirty = true;
    }
    return 0;
}

int tc_ensemble_get_schedule(const tc_ensemble* e) { return e ? e->schedule : -1; }

int tc_ensemble_set_barrier_timeout(tc_ensemble* e, double seconds) {
    if (!e) return 2000;
    if (!(seconds > 0.0) || seconds > 3600.0) return efail(e, 2013, "barrier timeout must be in (0, 3600] s");
    e->barrier_timeout = seconds;
    e->dirty = true;                     // the timeout is an argument of the captured launches
    return 0;
}

int tc_ensemble_stall_next_barrier(tc_ensemble* e) {
    if (!e) return 2000;
    if (e->schedule != TC_SCHED_PERSISTENT) return efail(e, 2013, "the ensemble does not use the persistent schedule");
    if (int r = prepare(e)) return r;
    if (!e->bar) return efail(e, 2013, "the ensemble has no persistent barrier yet (no members)");
    // an arrival count that no number of arrivals brings to the grid size:
    // the next barrier's generation never changes and every wait runs out
    const unsigned stuck = 0x80000000u;
    cudaError_t c = cudaMemcpyAsync(e->bar, &stuck, sizeof stuck, cudaMemcpyHostToDevice, e->stream);
    if (c == cudaSuccess) c = e->stream ? cudaStreamSynchronize(e->stream) : cudaDeviceSynchronize();
    if (c != cudaSuccess) return ecuda(e, c, "barrier stall");
    return 0;
}

int tc_ensemble_persistent_blocks(const tc_ensemble* e) { return e ? e->persist_blocks : 0; }

int tc_ensemble_step(tc_ensemble* e, int nsteps) {
    if (!e) return 2000;
    if (int r = prepare(e)) return r;
    if (e->active.empty()) return 0;
    for (int n = 0; n < nsteps; ++n) {
        cudaError_t c = cudaGraphLaunch(e->exec, e->stream);
        if (c != cudaSuccess) return ecuda(e, c, "graph launch");
        e->launches += e->launches_per_step;
    }
    return 0;
}

int tc_ensemble_sync(tc_ensemble* e) {
    if (!e) return 2000;
    cudaError_t c = e->stream ? cudaStreamSynchronize(e->stream) : cudaDeviceSynchronize();
    if (c != cudaSuccess) return ecuda(e, c, "ensemble sync");
    return check_barrier(e);
}

int tc_ensemble_status(tc_ensemble* e, int slot, int* steps_done, double* time, double* dt, int* errorcode) {
    tc_handle* h = nullptr;
    if (int r = tc_ensemble_member(e, slot, &h)) return r;
    StepState st;
    cudaError_t c = cudaMemcpyAsync(&st, h->st, sizeof st, cudaMemcpyDeviceToHost, e->stream);
    if (c == cudaSuccess) c = e->stream ? cudaStreamSynchronize(e->stream) : cudaDeviceSynchronize();
    if (c != cudaSuccess) return ecuda(e, c, "status read");
    if (int r = check_barrier(e)) return r;
    if (steps_done) *steps_done = st.ntime;
    if (time) *time = st.time;
    if (dt) *dt = st.dt;
    if (errorcode) *errorcode = st.errorcode;
    return 0;
}

long long tc_ensemble_launch_count(const tc_ensemble* e) { return e ? e->launches : 0; }
int tc_ensemble_launches_per_step(const tc_ensemble* e) { return e ? e->launches_per_step : 0; }

long long tc_ensemble_device_bytes(const tc_ensemble* e) {
    if (!e) return 0;
    long long b = 0;
    for (tc_handle* h : e->members) if (h) b += tc_device_bytes(h);
    return b;
}

long long tc_ensemble_cells(const tc_ensemble* e) {
    if (!e) return 0;
    long long c = 0;
    for (int s : e->active) c += e->members[s]->d.P * e->members[s]->d.nr;
    return c;
}
