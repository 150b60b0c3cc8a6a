// tc_ens.cuh -- what the ensemble kernels share (tc_batch.cu: grouped launches
// per phase; tc_persist.cu: one persistent launch per substep): the
// per-member parameter block, the phase enumeration and the lookup of a work
// item's member in a prefix table of item counts.
#pragma once

#include "tc_bodies.cuh"

namespace tcgb {
namespace ens {

template <typename T>
struct InstT {
    Dims d;
    CoefT<T> cv;
    Coef c;
    Consts k;
    FieldsT<T> f;
    PlansT<T> p;
    MomArgs<T> ma[3];
    int vdt;          // 1: dt from the CFL number every step (main.F90:156-174); 0: fixed dt
    // grouped schedule: theta rows per block of the divergence + forward FFT
    // (rows = 2^lg_rows) and of the inverse FFT, per member
    int rows, lg_rows, rows_inv, lg_rows_inv;
};

enum { PH_MOM = 0, PH_RAD, PH_DIV, PH_ZFFT, PH_PTRI, PH_THINV, PH_CORR, PH_FACT, PH_CFL, PH_COUNT };

constexpr double kCflFloor = 0.00000001;   // CalcMaxCFL.F90 starts its maximum here

// Momentum work units of one radial level (FP64) or chunk of kMomChunk
// levels (FP32 march) of a member: theta-neighbouring cell pairs
// (momentum_pair, momentum_column_x2).
template <typename T>
__host__ __device__ __forceinline__ long long mom_units(long long P) { return P / 2; }

// Cell (i, j) of the first cell of momentum unit u of a member with nt
// theta cells (nt is even).
template <typename T>
__device__ __forceinline__ void mom_unit_cell(int u, int nt, int& i, int& j) {
    const int half = nt / 2;
    j = (int)((unsigned)u / (unsigned)half);
    i = 2 * (u - j * half);
}

// The momentum work of unit (i, j) at level/chunk `outer` of substep args ma.
template <typename T>
__device__ __forceinline__ void mom_unit(const Dims& d, const CoefT<T>& cv, const MomArgs<T>& ma, int i, int j,
                                         int outer) {
    if constexpr (MomMarch<T>::value) {
        const int k0 = outer * kMomChunk;
        momentum_column_x2(d, cv, ma, i, j, k0, min(k0 + kMomChunk, d.nr));
    } else {
        momentum_pair(d, cv, ma, i, j, outer);
    }
}

// Work units of one radial level of the projection and of one component of
// the radial sweeps: FP32 two theta-neighbouring cells / columns
// (correct_pair_f, radial_column_pair), FP64 one.
template <typename T>
__host__ __device__ __forceinline__ long long cell_units(long long P) {
    return std::is_same<T, float>::value ? P / 2 : P;
}

// The projection of unit u at level k.
template <typename T>
__device__ __forceinline__ void corr_unit(const Dims& d, const FieldsT<T>& f, int sub, int u, int k) {
    if constexpr (std::is_same<T, float>::value) {
        int i, j;
        mom_unit_cell<T>(u, d.nt, i, j);
        correct_pair_f(d, f, sub, i, j, k);
    } else {
        const int j = (int)((unsigned)u / (unsigned)d.nt), i = u - j * d.nt;
        correct_cell<true, true, T>(d, f, sub, i, j, k);
    }
}

// The radial sweep of unit u for component comp.
template <typename T>
__device__ __forceinline__ void rad_unit(const Dims& d, const FieldsT<T>& f, int sub, long long u, int comp) {
    if constexpr (std::is_same<T, float>::value) radial_column_pair(d, f, sub, 2 * u, comp);
    else radial_column(d, f, sub, u, comp);
}

__device__ __forceinline__ int find_member(const int* prefix, int n, long long item) {
    int lo = 0, hi = n;
    while (hi - lo > 1) {
        int mid = (lo + hi) >> 1;
        if (prefix[mid] <= item) lo = mid;
        else hi = mid;
    }
    return lo;
}

// The persistent schedule: one cooperative launch per RK substep.  The
// first substep's launch also reduces the CFL numbers of variable-dt members,
// sets each member's dt, beta and inner-wall forcing and factors the momentum
// matrices; the last one also advances time.  Between phases the blocks meet
// at a grid-wide barrier.  Tables are those of the grouped kernels, built
// with kPersistThreads threads per tile and R <= kPersistMaxRows rows per
// theta-FFT item.
constexpr int kPersistThreads = 128;
constexpr int kPersistMaxRows = 8;

enum { PF_CFL = 1, PF_BEGIN = 2, PF_FACT = 4, PF_END = 8 };

struct PersistArgs {
    const int* prefix;           // PH_COUNT tables of n + 1 entries
    int n;
    int items[PH_COUNT];
    int sub;
    int flags;                   // PF_* phases around the substep
    unsigned* bar_count;         // barrier arrival counter (0 between barriers)
    unsigned* bar_gen;           // barrier generation
    int* err;                    // set to 1 when a barrier wait gives up
    unsigned long long timeout_ns;   // bound on one barrier wait (device global timer)
};

// Blocks of the persistent kernel for R rows and `smem` bytes of dynamic
// shared memory: SMs x the occupancy limit, or x per_sm_cap if that is
// smaller and positive (fewer blocks: cheaper barriers, fewer warps).  Sets
// the kernel's shared memory attribute; call outside stream capture.
template <typename T>
cudaError_t prepare_persistent(int R, size_t smem, int per_sm_cap, int* blocks);

// Enqueue one persistent substep on `s` (cooperative launch of `blocks`
// blocks, as prepare_persistent returned); returns the launch's status.
template <typename T>
cudaError_t launch_persistent(cudaStream_t s, const InstT<T>* inst, const PersistArgs& a, int R, size_t smem,
                              int blocks);

}  // namespace ens
}  // namespace tcgb
