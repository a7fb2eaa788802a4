// bk_internal.h -- declarations shared by the translation units of the
// library (not part of the C ABI).
#pragma once

#include <cuda_runtime.h>

#include "bk_gpu.h"

namespace bkg {

struct DevCtx;

constexpr int kMaxDevices = 64;

int current_device();          // cudaGetDevice, or -1

// BK5's built-in choice for BK_KERNEL_AUTO (measured on GB300 at about 2^24
// DoFs, mixed form, GDoF/s sweep / column): the column kernel for the
// FP32-storage engines (2: FP32, 3: mixed) with G in the column layout at
// p <= 3 (p = 1..3: 100 / 129, 116 / 126, 167 / 174) and at p = 5 with the
// mass term (131 / 135), the sweep kernel otherwise (p = 4 141 / 138, p = 5
// without the mass term 147 / 144, p >= 6 by 19-83 %).
inline int bk5_builtin_auto(int p, int eng, int layout, bool with_mass)
{
    return (eng >= 2 && layout == 2 && (p <= 3 || (p == 5 && with_mass))) ? BK_KERNEL_COLUMN : BK_KERNEL_SWEEP;
}
int sm_count();                // SMs of the current device
DevCtx dev_ctx();              // status word and wait limit of the current device

#define BK_DECLARE_ENGINE(sfx)                                                                                    \
    int launch_bk5_##sfx(int p, long long E, const double* D, const void* G, const void* u, const void* mass,    \
                         double lambda, void* v, int F, int layout, int eb, int kernel, int gform, cudaStream_t s); \
    int launch_bk1_##sfx(int p, long long E, const double* B, const void* jxw, const void* u, void* v, int eb,   \
                         int jxw_t, cudaStream_t s);                                                             \
    int launch_bk3_##sfx(int p, long long E, const double* B, const double* D, const void* G, const void* k,     \
                         const void* u, void* v, int eb, int gform, cudaStream_t s);                                        \
    int bk5_sweep_##sfx##_L0(int p, int F, const double* D, long long E, const void* u, const void* G,  \
                             const void* mass, double lambda, void* v, int gform, cudaStream_t s);                          \
    int bk5_sweep_##sfx##_L1(int p, int F, const double* D, long long E, const void* u, const void* G,  \
                             const void* mass, double lambda, void* v, int gform, cudaStream_t s);                          \
    int bk5_sweep_##sfx##_L2(int p, int F, const double* D, long long E, const void* u, const void* G,  \
                             const void* mass, double lambda, void* v, int gform, cudaStream_t s);                               \
    int bk5_col_##sfx##_L0(int p, int F, int eb, const double* D, long long E, const void* u, const void* G,    \
                           const void* mass, double lambda, void* v, cudaStream_t s);                            \
    int bk5_col_##sfx##_L1(int p, int F, int eb, const double* D, long long E, const void* u, const void* G,    \
                           const void* mass, double lambda, void* v, cudaStream_t s);                            \
    int launch_bk3_adjoint_##sfx(int p, long long E, const double* B, const double* D, const void* G,           \
                                 const void* k, const void* u, const void* res, void* dk, void* dG,              \
                                 int gform, cudaStream_t s);                                                                \
    int bk5_col_##sfx##_L2(int p, int F, int eb, const double* D, long long E, const void* u, const void* G,    \
                           const void* mass, double lambda, void* v, cudaStream_t s);

BK_DECLARE_ENGINE(dfma)
BK_DECLARE_ENGINE(ff)
BK_DECLARE_ENGINE(f32)
BK_DECLARE_ENGINE(mixed)

}  // namespace bkg
