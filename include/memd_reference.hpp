// memd_reference.hpp -- the reference's C++ entry points, implemented over the
// C ABI of libmemd_gb300.so, so a program written against
// memReducedEpochs_dev.cu compiles and links unchanged (header-only).
//
//   template<coord_t, real_t> double memd(size_t SignalDim, size_t SignalLength,
//       size_t NumDirVector, size_t num_IMFs, size_t max_iter, coord_t* d_x,
//       real_t* d_y, real_t* d_DirectionVectors, real_t* d_IMFs)
//                                        memReducedEpochs_dev.cu:1074-1075
//   template<T> void GenerateDirectionVector(size_t SignalDim,
//       size_t NumDirVector, T* d_DirectionVector)
//                                        memReducedEpochs_dev.cu:1029-1030
//
// Same arguments, same device layouts (d_y: SignalDim x SignalLength
// channel-major; directions NumDirVector x SignalDim; d_IMFs num_IMFs x
// SignalDim x SignalLength with the residual in the last slot), same return
// value: the seconds spent in the decomposition (the reference times its IMF
// loop with omp_get_wtime, REF:1175 and 1336-1337; here CUDA events around the
// decomposition graph, allocation excluded in both).  real_t = double runs the
// FP64 path, real_t = float the FP32 path (the reference's own precision);
// define MEMD_FLOAT_FORM_MIXED before including to run float inputs through
// the mixed-precision form instead.
//
// Differences a caller may notice: errors are reported (the reference reports
// none): on failure memd() prints the reason to stderr and returns -1.0; and
// the workspace is allocated once and reused while the sizes stay the same
// (the reference allocates and frees it on every call).
#ifndef MEMD_REFERENCE_HPP
#define MEMD_REFERENCE_HPP

#include <cstddef>
#include <cstdint>
#include <cstdio>
#include <type_traits>

#include "memd_gb300.h"

namespace memd_detail {

struct PlanCache {
    memd_plan* plan = nullptr;
    memd_config cfg{};
    ~PlanCache()
    {
        if (plan) memd_plan_destroy(plan);
    }
    memd_plan* get(const memd_config& c)
    {
        if (plan && cfg.channels == c.channels && cfg.length == c.length && cfg.directions == c.directions &&
            cfg.num_imfs == c.num_imfs && cfg.max_iter == c.max_iter && cfg.precision == c.precision)
            return plan;
        if (plan) memd_plan_destroy(plan);
        plan = nullptr;
        if (memd_plan_create(&c, &plan) != MEMD_OK) {
            std::fprintf(stderr, "memd: plan creation failed: %s\n", memd_last_error());
            plan = nullptr;
            return nullptr;
        }
        cfg = c;
        return plan;
    }
};

inline PlanCache& cache()
{
    static thread_local PlanCache c;
    return c;
}

}  // namespace memd_detail

template <typename T>
void GenerateDirectionVector(size_t SignalDim, size_t NumDirVector, T* d_DirectionVector)
{
    static_assert(std::is_same<T, float>::value || std::is_same<T, double>::value,
                  "GenerateDirectionVector: float or double");
    memd_status st;
    if (std::is_same<T, double>::value)
        st = memd_directions_f64((int64_t)SignalDim, (int64_t)NumDirVector, nullptr,
                                 reinterpret_cast<double*>(d_DirectionVector), nullptr);
    else
        st = memd_directions_f32((int64_t)SignalDim, (int64_t)NumDirVector, nullptr,
                                 reinterpret_cast<float*>(d_DirectionVector), nullptr);
    if (st != MEMD_OK) std::fprintf(stderr, "GenerateDirectionVector: %s\n", memd_last_error());
}

template <typename coord_t, typename real_t>
double memd(size_t SignalDim, size_t SignalLength, size_t NumDirVector, size_t num_IMFs, size_t max_iter,
            coord_t* d_x, real_t* d_y, real_t* d_DirectionVectors, real_t* d_IMFs)
{
    static_assert(sizeof(coord_t) == 4 && std::is_integral<coord_t>::value, "memd: coord_t must be a 32-bit integer");
    static_assert(std::is_same<real_t, float>::value || std::is_same<real_t, double>::value,
                  "memd: real_t must be float or double");
    memd_config cfg;
    memd_default_config(&cfg);
    cfg.channels = (int64_t)SignalDim;
    cfg.length = (int64_t)SignalLength;
    cfg.directions = (int64_t)NumDirVector;
    cfg.num_imfs = (int64_t)num_IMFs;
    cfg.max_iter = (int64_t)max_iter;
#ifdef MEMD_FLOAT_FORM_MIXED
    cfg.precision = std::is_same<real_t, double>::value ? MEMD_PREC_F64 : MEMD_PREC_MIXED;
#else
    cfg.precision = std::is_same<real_t, double>::value ? MEMD_PREC_F64 : MEMD_PREC_F32;
#endif
    memd_plan* plan = memd_detail::cache().get(cfg);
    if (!plan) return -1.0;
    memd_stats stats;
    memd_status st;
    if (std::is_same<real_t, double>::value)
        st = memd_run_f64(plan, reinterpret_cast<const int32_t*>(d_x), reinterpret_cast<const double*>(d_y),
                          reinterpret_cast<const double*>(d_DirectionVectors), reinterpret_cast<double*>(d_IMFs),
                          nullptr, &stats);
    else
        st = memd_run_f32(plan, reinterpret_cast<const int32_t*>(d_x), reinterpret_cast<const float*>(d_y),
                          reinterpret_cast<const float*>(d_DirectionVectors), reinterpret_cast<float*>(d_IMFs),
                          nullptr, &stats);
    if (st != MEMD_OK) {
        std::fprintf(stderr, "memd: %s\n", memd_last_error());
        return -1.0;
    }
    return stats.elapsed_ms * 1e-3;
}

#endif  // MEMD_REFERENCE_HPP
