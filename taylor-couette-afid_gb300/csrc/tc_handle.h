// tc_handle.h -- the handle behind the C ABI (one simulation instance).
#pragma once

#include <string>
#include <vector>

#include "../../include/tc_capi.h"
#include "tc_grid.h"
#include "tc_kernels.cuh"

struct tc_handle {
    tc_bou bou;
    int mixed = 0;          // 0: plain FP64, 1: mixed FP32/FP64
    int ptri_ff = 0;        // mixed: pressure tridiagonals in float-float instead of FP64
    tcgb::Grid g;
    tcgb::Dims d;
    tcgb::Consts k;
    tcgb::Coef c;                 // FP64 coefficients (pressure, reductions, factors)
    tcgb::CoefT<float> cf;        // FP32 copies (mixed path velocity kernels)
    tcgb::FieldsT<double> fd;     // plain path state
    tcgb::FieldsT<float> ff;      // mixed path state
    tcgb::PlansT<double> pd;
    tcgb::PlansT<float> pf;
    tcgb::MarchMaps maps;         // TMA descriptors of the mixed march (ff.tma points here when in use)
    bool maps_ok = false;
    cudaStream_t stream = nullptr;
    std::vector<void*> allocs;
    double* stage = nullptr;
    tcgb::StepState* st = nullptr;        // device
    tcgb::StepState* st_host = nullptr;   // pinned mirror
    int sub = 0;
    long long bytes = 0;
    std::string err;
    // launch accounting and optional per-kernel event timing
    long long launches = 0;
    bool profiling = false;
    struct Rec { int cls; cudaEvent_t a, b; };
    std::vector<Rec> recs;
    std::vector<cudaEvent_t> pool;
    size_t pool_used = 0;
    double prof_ms[16] = {0};
    long long prof_n[16] = {0};
    // statistics (StatRoutines.F90 stat_arrays), allocated at the first use:
    // TC_ST_COUNT arrays of (nrm, nzm), r fastest, plus per-row dissipation
    double* stats = nullptr;
    double* stat_rows = nullptr;
    int nstatsamples = 0;
};
