// tc_persist.cu -- the persistent schedule of an ensemble: one cooperative
// launch per RK substep runs every phase of the substep for every member,
// with grid-wide barriers between the phases (tc_ens.cuh).
//
// The blocks of a cooperative launch are all resident at once; in each phase
// they stride over the phase's flat work list of (member, tile) items and run
// the same device bodies as the grouped kernels of tc_batch.cu, so a member's
// arithmetic does not depend on the schedule.
//
// Loads: a phase reads what other blocks wrote in an earlier phase of the
// same launch, so this file defines TC_COHERENT_LOADS, which makes the
// bodies' field loads ordinary (coherent) global loads instead of loads
// through the read-only path.  The barrier orders the phases: every block
// fences its writes before it arrives and fences again after it sees the
// generation change.
//
// The barrier waits are bounded: a block whose wait has lasted timeout_ns
// (device global timer; kBarrierPolls polls at most) records 1 in *err and
// leaves at that barrier; a block finding *err set leaves at its next
// barrier, and a launch that starts with *err set does nothing.  The host
// reads *err when it synchronises (tc_ensemble_sync) and resets the barrier.

#define TC_COHERENT_LOADS 1
#include "tc_ens.cuh"

namespace tcgb {
namespace ens {
namespace {

constexpr long long kBarrierPolls = 1LL << 26;

__device__ __forceinline__ unsigned long long global_ns() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

__device__ bool grid_barrier(const PersistArgs& a) {
    __shared__ int ok;
    __syncthreads();
    if (threadIdx.x == 0) {
        int good = 1;
        volatile unsigned* gen = a.bar_gen;
        const unsigned g = *gen;
        __threadfence();
        const unsigned arrived = atomicAdd(a.bar_count, 1u) + 1u;
        if (arrived == gridDim.x) {
            atomicExch(a.bar_count, 0u);
            __threadfence();
            atomicAdd(a.bar_gen, 1u);
        } else {
            const unsigned long long t0 = global_ns();
            long long polls = 0;
            while (*gen == g) {
                if (++polls > kBarrierPolls || global_ns() - t0 > a.timeout_ns) {
                    atomicExch(a.err, 1);
                    good = 0;
                    break;
                }
                __nanosleep(200);
            }
        }
        __threadfence();
        if (*(volatile int*)a.err) good = 0;
        ok = good;
    }
    __syncthreads();
    return ok != 0;
}

// Cell tile of a (level or chunk, tile) item: the flat (j, i) index of this
// thread and the level/chunk/component of the item.
struct CellItem {
    int outer;
    long long flat;
};
__device__ __forceinline__ CellItem cell_item(long long local, size_t P) {
    const int tiles = (int)((P + kPersistThreads - 1) / kPersistThreads);
    CellItem c;
    c.outer = (int)((unsigned)local / (unsigned)tiles);
    c.flat = (local - (long long)c.outer * tiles) * kPersistThreads + threadIdx.x;
    return c;
}

template <int R, typename T>
__global__ void __launch_bounds__(kPersistThreads) persist_kernel(const InstT<T>* __restrict__ inst, PersistArgs a) {
    typedef typename V2<T>::type C2;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    C2* smem = reinterpret_cast<C2*>(smem_raw);
    __shared__ double red[kPersistThreads / 32];
    const int n = a.n, sub = a.sub;
    constexpr int ZC = ZCols<T>::value;
    auto table = [&](int ph) { return a.prefix + (size_t)ph * (n + 1); };
    const long long gthreads = (long long)gridDim.x * kPersistThreads;
    const long long gtid = (long long)blockIdx.x * kPersistThreads + threadIdx.x;

    if (*(volatile int*)a.err) return;   // an earlier launch gave up at a barrier

    if (a.flags & PF_CFL) {
        // CalcMaxCFL of the variable-dt members: block maximum over a
        // (level, tile) item, then an atomic maximum on the bits of the
        // member's instcfl (non-negative doubles order as their bits)
        for (long long item = blockIdx.x; item < a.items[PH_CFL]; item += gridDim.x) {
            const int m = find_member(table(PH_CFL), n, item);
            const InstT<T>& I = inst[m];
            if (I.f.st->halt) continue;
            const CellItem ci = cell_item(item - table(PH_CFL)[m], I.d.P);
            double v = 0.0;
            if (ci.flat < (long long)I.d.P) {
                const int j = (int)((unsigned)ci.flat / (unsigned)I.d.nt), i = (int)ci.flat - j * I.d.nt;
                v = cfl_cell(I.d, I.c, I.cv, I.k.dxt, I.k.dxz, I.f, i, j, ci.outer);
            }
            for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, o));
            const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
            if (l == 0) red[w] = v;
            __syncthreads();
            if (w == 0) {
                v = (l < kPersistThreads / 32) ? red[l] : 0.0;
                for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, o));
                if (l == 0)
                    atomicMax(reinterpret_cast<unsigned long long*>(&I.f.st->instcfl),
                              (unsigned long long)__double_as_longlong(v));
            }
            __syncthreads();
        }
        if (!grid_barrier(a)) return;
    }
    if (a.flags & PF_BEGIN) {
        // dt, beta and inner-wall forcing per member (as ens_begin_kernel)
        for (long long m = gtid; m < n; m += gthreads) {
            StepState* st = inst[m].f.st;
            if (!st->halt) begin_step_body(inst[m].k, st, inst[m].vdt, st->dt, st->time);
        }
        if (!grid_barrier(a)) return;
    }
    if (a.flags & PF_FACT) {
        // factors of this step's momentum matrices, one block per member
        for (long long item = blockIdx.x; item < a.items[PH_FACT]; item += gridDim.x) {
            const InstT<T>& I = inst[item];
            if (!I.f.st->halt) factors_body(I.d, I.c, I.k, I.f.st, I.f.Fd, I.f.corrd, I.f.scal, I.f.F, I.f.corr);
            __syncthreads();
        }
        if (!grid_barrier(a)) return;
    }
    // momentum: (chunk of kMomChunk levels, tile of theta-neighbouring column
    // pairs) marching in r; for FP64 (level, tile of cell pairs)
    for (long long item = blockIdx.x; item < a.items[PH_MOM]; item += gridDim.x) {
        const int m = find_member(table(PH_MOM), n, item);
        const InstT<T>& I = inst[m];
        if (I.f.st->halt) continue;
        const long long units = mom_units<T>(I.d.P);
        const CellItem ci = cell_item(item - table(PH_MOM)[m], (size_t)units);
        if (ci.flat < units) {
            int i, j;
            mom_unit_cell<T>((int)ci.flat, I.d.nt, i, j);
            mom_unit(I.d, I.cv, I.ma[sub], i, j, ci.outer);
        }
    }
    if (!grid_barrier(a)) return;
    // radial solves: (component, tile of columns)
    for (long long item = blockIdx.x; item < a.items[PH_RAD]; item += gridDim.x) {
        const int m = find_member(table(PH_RAD), n, item);
        const InstT<T>& I = inst[m];
        if (I.f.st->halt) continue;
        const long long units = cell_units<T>(I.d.P);
        const CellItem ci = cell_item(item - table(PH_RAD)[m], (size_t)units);
        if (ci.flat < units) rad_unit(I.d, I.f, sub, ci.flat, ci.outer);
    }
    if (!grid_barrier(a)) return;
    // divergence + theta FFT: R rows per item
    for (long long item = blockIdx.x; item < a.items[PH_DIV]; item += gridDim.x) {
        const int m = find_member(table(PH_DIV), n, item);
        const InstT<T>& I = inst[m];
        if (!I.f.st->halt)
            div_fft_rows<false, R, T>(I.d, I.cv, (T)I.k.dxt, (T)I.k.dxz, I.f, I.p.th, I.p.tw_th, I.p.twr,
                                      I.k.fft_norm, sub, (item - table(PH_DIV)[m]) * R, smem);
        __syncthreads();
    }
    if (!grid_barrier(a)) return;
    for (int inv = 0; inv < 2; ++inv) {
        // z FFT, forward and (after the tridiagonals) inverse: ZC columns of a plane
        for (long long item = blockIdx.x; item < a.items[PH_ZFFT]; item += gridDim.x) {
            const int m = find_member(table(PH_ZFFT), n, item);
            const InstT<T>& I = inst[m];
            if (!I.f.st->halt) {
                const int local = (int)(item - table(PH_ZFFT)[m]);
                const int groups = (I.d.PH + ZC - 1) / ZC;
                const int kplane = local / groups, g = local - kplane * groups;
                zfft_tile<ZC>(I.d, I.f, I.p.z, I.p.tw_z, inv, g * ZC, kplane, smem);
            }
            __syncthreads();
        }
        if (!grid_barrier(a)) return;
        if (inv) break;
        // pressure tridiagonals: one (kz, kt) mode per thread
        for (long long item = blockIdx.x; item < a.items[PH_PTRI]; item += gridDim.x) {
            const int m = find_member(table(PH_PTRI), n, item);
            const InstT<T>& I = inst[m];
            if (I.f.st->halt) continue;
            const long long t = (item - table(PH_PTRI)[m]) * kPersistThreads + threadIdx.x;
            if (t < (long long)I.d.nz * I.d.PH) {
                ptri_solve(I.d, I.c, I.f, t);
            }
        }
        if (!grid_barrier(a)) return;
    }
    // inverse theta FFT: R rows per item
    for (long long item = blockIdx.x; item < a.items[PH_THINV]; item += gridDim.x) {
        const int m = find_member(table(PH_THINV), n, item);
        const InstT<T>& I = inst[m];
        if (!I.f.st->halt)
            thinv_rows<R, T>(I.d, I.f, I.p.th, I.p.tw_th, I.p.twr, (item - table(PH_THINV)[m]) * R, smem);
        __syncthreads();
    }
    if (!grid_barrier(a)) return;
    // correction: (level, tile of cells)
    for (long long item = blockIdx.x; item < a.items[PH_CORR]; item += gridDim.x) {
        const int m = find_member(table(PH_CORR), n, item);
        const InstT<T>& I = inst[m];
        if (I.f.st->halt) continue;
        const long long units = cell_units<T>(I.d.P);
        const CellItem ci = cell_item(item - table(PH_CORR)[m], (size_t)units);
        if (ci.flat < units) corr_unit(I.d, I.f, sub, (int)ci.flat, ci.outer);
    }
    if (a.flags & PF_END) {
        if (!grid_barrier(a)) return;
        // time = time + dt (as ens_end_kernel)
        for (long long m = gtid; m < n; m += gthreads) {
            StepState* st = inst[m].f.st;
            if (st->halt) continue;
            st->time = st->time + st->dt;
            st->ntime += 1;
            if (st->errorcode != 0) st->halt = 1;
            st->instcfl = kCflFloor;
        }
    }
}

template <typename T>
void* persist_fn(int R) {
    switch (R) {
        case 1: return (void*)persist_kernel<1, T>;
        case 2: return (void*)persist_kernel<2, T>;
        case 4: return (void*)persist_kernel<4, T>;
        default: return (void*)persist_kernel<8, T>;
    }
}

}  // namespace

template <typename T>
cudaError_t prepare_persistent(int R, size_t smem, int per_sm_cap, int* blocks) {
    const void* fn = persist_fn<T>(R);
    cudaError_t c = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (c != cudaSuccess) return c;
    int dev = 0, sms = 0, per = 0;
    if ((c = cudaGetDevice(&dev)) != cudaSuccess) return c;
    if ((c = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev)) != cudaSuccess) return c;
    if ((c = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, fn, kPersistThreads, smem)) != cudaSuccess) return c;
    if (per < 1) return cudaErrorInvalidConfiguration;
    if (per_sm_cap > 0 && per_sm_cap < per) per = per_sm_cap;
    *blocks = sms * per;
    return cudaSuccess;
}

template <typename T>
cudaError_t launch_persistent(cudaStream_t s, const InstT<T>* inst, const PersistArgs& a, int R, size_t smem,
                              int blocks) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((unsigned)blocks);
    cfg.blockDim = dim3(kPersistThreads);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = s;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeCooperative;
    attr[0].val.cooperative = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    void* args[] = {(void*)&inst, (void*)&a};
    return cudaLaunchKernelExC(&cfg, persist_fn<T>(R), args);
}

template cudaError_t prepare_persistent<double>(int, size_t, int, int*);
template cudaError_t prepare_persistent<float>(int, size_t, int, int*);
template cudaError_t launch_persistent<double>(cudaStream_t, const InstT<double>*, const PersistArgs&, int, size_t,
                                               int);
template cudaError_t launch_persistent<float>(cudaStream_t, const InstT<float>*, const PersistArgs&, int, size_t,
                                              int);

}  // namespace ens
}  // namespace tcgb
