// bk_ops.cu -- launchers of the BK1 / BK3 / BK5 kernels for ONE arithmetic
// engine, chosen at compile time by BK_ENGINE_TU (0 dfma, 1 float-float,
// 2 fp32, 3 mixed): the build compiles this file once per engine so that the
// translation units build in parallel.  Run-time order p -> compile-time Q
// (the role of bk::with_order, include/bk_common.h:148-178).
#include <cuda_runtime.h>

#include "bk_internal.h"
#include "bk5_col.cuh"
#include "bk_adjoint.cuh"
#include "bk_kernels.cuh"

#ifndef BK_ENGINE_TU
#error "BK_ENGINE_TU must be 0 (dfma), 1 (ff), 2 (fp32) or 3 (mixed)"
#endif
// BK_OP_TU selects the operator of this translation unit: 1 BK1, 3 BK3,
// 5 BK5 sweep kernel and 6 BK5 column kernel (one G layout each,
// BK_LAYOUT_TU), 7 the BK3 adjoint and the BK5 dispatch.
#ifndef BK_OP_TU
#error "BK_OP_TU must be 1, 3, 5, 6 or 7"
#endif

namespace bkg {

#if BK_ENGINE_TU == 0
using Eng = EngDfma;
#define BK_SFX dfma
#elif BK_ENGINE_TU == 1
using Eng = EngFF;
#define BK_SFX ff
#elif BK_ENGINE_TU == 2
using Eng = EngF32;
#define BK_SFX f32
#else
using Eng = EngMixed;
#define BK_SFX mixed
#endif

#define BK_CAT2(a, b) a##_##b
#define BK_CAT(a, b) BK_CAT2(a, b)

#ifndef BK_LAYOUT_TU
#define BK_LAYOUT_TU 9
#endif
// A namespace of its own per translation unit: every unit compiles this file,
// and nvcc may give an anonymous namespace the same name in all of them, so
// same-named helpers of different engines or layouts would be merged (or
// clash) at link time.
#define BK_NS3_(a, b, c) tu_##a##_##b##_##c
#define BK_NS3(a, b, c) BK_NS3_(a, b, c)
#define BK_TU_NS BK_NS3(BK_ENGINE_TU, BK_OP_TU, BK_LAYOUT_TU)

namespace BK_TU_NS {

// Elements per block: about 128 lines per sweep (Q^2 lines per element).
constexpr int default_eb(int q) { return (q * q >= 100) ? 1 : ((q * q >= 64) ? 2 : (128 + q * q - 1) / (q * q)); }

// Elements per block of the BK5 and BK3 sweep kernels (even-odd path), the
// fastest of EB = 1..16 measured per engine and q on GB300 (about 2^24 DoFs
// per apply).  Small orders want many elements per block (short lines, small
// boxes); from q = 8 one element per block, whose smaller shared-memory
// footprint keeps more blocks resident, wins for the FP32-pipe engines.
constexpr bool eng_is_dfma() { return Eng::kId == BK_ENGINE_DFMA; }
constexpr bool eng_is_ff() { return Eng::kId == BK_ENGINE_FF; }
constexpr int sweep_eb5(int q)
{
    if (q <= 3) return eng_is_ff() || eng_is_dfma() ? 16 : 12;
    if (q == 4) return 8;
    if (eng_is_dfma()) return q == 5 ? 6 : q == 6 ? 4 : q == 7 ? 3 : q == 8 ? 2 : 3;
    if (eng_is_ff()) return q == 5 ? 4 : q == 6 ? 3 : q == 7 ? 4 : 1;
    return q == 5 ? 4 : q == 6 ? 3 : q == 7 ? 2 : 1;
}
constexpr int sweep_eb3(int q)
{
    if (q <= 3) return eng_is_ff() ? 12 : 16;
    if (q == 4) return 8;
    if (eng_is_dfma()) return q == 5 ? 6 : q == 6 ? 4 : q == 7 ? 3 : q == 8 ? 2 : q == 9 ? 3 : 1;
    if (eng_is_ff()) return q == 5 ? 8 : q <= 7 ? 3 : 1;
    return q == 5 ? 6 : q == 6 ? 4 : q == 7 ? 3 : 1;
}

// Sets the dynamic shared-memory size of a kernel on the current device once
// and returns its resident blocks per SM (0 if it cannot run).  Tag makes the
// cache one per kernel instantiation (kernels of one signature share K).
template <class Cfg, bool EO>
struct EoTag {};

template <class Tag, class K>
int prepare(K kern, int smem, int nt)
{
    static int occ[kMaxDevices] = {0};
    const int dev = current_device();
    if (dev < 0 || dev >= kMaxDevices) return 0;
    if (occ[dev] == 0) {
        if (cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, smem) != cudaSuccess) return 0;
        int n = 0;
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, kern, nt, smem) != cudaSuccess) return 0;
        occ[dev] = n;
    }
    return occ[dev];
}

int grid_for(long long nbatch, int occ)
{
    const long long cap = static_cast<long long>(occ) * sm_count();
    return static_cast<int>(nbatch < cap ? nbatch : cap);
}

#if BK_OP_TU == 5
// One launch of bk5_kernel with the given shape.
// GS: the type G is stored in (the storage type, or ff2 pairs split ahead of
// time for the float-float engine).
template <int Q, int EB, int F, int LAYOUT, bool EO, int DPAR, class GS = typename Eng::S>
int bk5_launch(const P5<typename Eng::C, Q>& prm, long long E, const void* u, const void* G, const void* mass,
               double lambda, void* v, cudaStream_t s)
{
    using Cfg = BK5Cfg<Eng, Q, EB, F, LAYOUT, DPAR>;
    using S = typename Eng::S;
    static_assert(Cfg::SMEM <= 232448, "BK5 block exceeds the shared memory of an SM");
    auto kern = bk5_kernel<Eng, Q, EB, F, LAYOUT, EO, DPAR, GS>;
    const int occ = prepare<EoTag<Cfg, EO>>(kern, Cfg::SMEM, Cfg::NT);
    if (occ <= 0) return BK_ERR_CUDA;
    const int grid = grid_for((E + EB - 1) / EB, occ);
    kern<<<grid, Cfg::NT, Cfg::SMEM, s>>>(prm, E, static_cast<const S*>(u), static_cast<const GS*>(G),
                                          static_cast<const S*>(mass), lambda, static_cast<S*>(v), dev_ctx());
    return cudaGetLastError() == cudaSuccess ? BK_OK : BK_ERR_CUDA;
}

// the largest EB <= EB0 whose block fits an SM's shared memory
template <int Q, int F, int EB0, int DPAR = 0>
constexpr int fit_eb5()
{
    if constexpr (EB0 > 1 && BK5Cfg<Eng, Q, EB0, F, BK_LAYOUT_TU, DPAR>::SMEM > 232448)
        return fit_eb5<Q, F, EB0 - 1, DPAR>();
    else
        return EB0;
}

// The direction-parallel even-odd shape (three thread groups, one direction
// each, one shared code body: DPAR = 2) for the float-float engine where it
// measured faster on GB300: q = 6 (EB 4), 7 (EB 2), 8 (EB 1) and 9 (EB 3),
// 2-33 % over one thread per line (q = 8: 36.9 against 30.2 GDoF/s).
constexpr bool sweep_dpar5(int q) { return eng_is_ff() && q >= 6 && q <= 9; }
constexpr int sweep_eb5_dpar(int q) { return q == 6 ? 4 : q == 7 ? 2 : q == 9 ? 3 : 1; }

template <int Q>
int bk5_sweep_q(int F, const double* D, long long E, const void* u, const void* G, const void* mass,
                double lambda, void* v, int gform, cudaStream_t s)
{
    constexpr int L = BK_LAYOUT_TU;
    P5<typename Eng::C, Q> prm;
    for (int i = 0; i < Q * Q; ++i) prm.D[i] = Eng::coef(D[i]);
    // the even-odd contractions when D is centro-antisymmetric (GLL points);
    // instantiated for the symmetric 6-factor G only
    const bool eo = (F == 6) && make_eo<typename Eng::C, Q>(D, false, prm.eo, &Eng::coef) &&
                    make_eo<typename Eng::C, Q>(D, true, prm.eot, &Eng::coef);
    if (eo) {
        constexpr int DP = sweep_dpar5(Q) ? 2 : 0;
        constexpr int EB = fit_eb5<Q, 6, DP ? sweep_eb5_dpar(Q) : sweep_eb5(Q), DP>();
        if (gform == BK_G_FF) {
            // G split ahead of time: the float-float engine's even-odd path
            if constexpr (eng_is_ff()) return bk5_launch<Q, EB, 6, L, true, DP, ff2>(prm, E, u, G, mass, lambda, v, s);
            return BK_ERR_PREC;
        }
        return bk5_launch<Q, EB, 6, L, true, DP>(prm, E, u, G, mass, lambda, v, s);
    }
    if (gform != BK_G_STORAGE) return BK_ERR_PREC;   // split G: even-odd D (GLL points), 6 factors
    if (F == 6) return bk5_launch<Q, fit_eb5<Q, 6, sweep_eb5(Q)>(), 6, L, false, 0>(prm, E, u, G, mass, lambda, v, s);
    if (F == 9) return bk5_launch<Q, fit_eb5<Q, 9, sweep_eb5(Q)>(), 9, L, false, 0>(prm, E, u, G, mass, lambda, v, s);
    return BK_ERR_PREC;
}
#endif  // BK_OP_TU == 5

#if BK_OP_TU == 6
// Column kernel: elements per block and stage buffers.  The FP32-storage
// forms are HBM-bound (double buffering), the FP64 engines ALU-bound (one
// stage, more blocks per SM).
constexpr int col_nbuf() { return (sizeof(typename Eng::S) == 4) ? 2 : 1; }
constexpr int col_eb(int q) { return (q * q >= 64) ? ((sizeof(typename Eng::S) == 4) ? 2 : 1) : (128 + q * q - 1) / (q * q); }

template <int Q, int EB, int F, int LAYOUT, int NBUF>
int bk5col_q(const double* D, long long E, const void* u, const void* G, const void* mass, double lambda, void* v,
             cudaStream_t s)
{
    using Cfg = BK5ColCfg<Eng, Q, EB, F, NBUF, LAYOUT>;
    using S = typename Eng::S;
    static_assert(Cfg::SMEM <= 232448, "BK5 block exceeds the shared memory of an SM");
    P5<typename Eng::C, Q> prm;
    for (int i = 0; i < Q * Q; ++i) prm.D[i] = Eng::coef(D[i]);
    auto kern = bk5_col_kernel<Eng, Q, EB, F, LAYOUT, NBUF>;
    const int occ = prepare<Cfg>(kern, Cfg::SMEM, Cfg::NT);
    if (occ <= 0) return BK_ERR_CUDA;
    const int grid = grid_for((E + EB - 1) / EB, occ);
    kern<<<grid, Cfg::NT, Cfg::SMEM, s>>>(prm, E, static_cast<const S*>(u), static_cast<const S*>(G),
                                          static_cast<const S*>(mass), lambda, static_cast<S*>(v), dev_ctx());
    return cudaGetLastError() == cudaSuccess ? BK_OK : BK_ERR_CUDA;
}

template <int Q>
int bk5col_f(int F, int eb, const double* D, long long E, const void* u, const void* G, const void* mass,
             double lambda, void* v, cudaStream_t s)
{
    constexpr int NB = col_nbuf();
    constexpr int EB0 = col_eb(Q);
    if (eb != 0 && eb != EB0) return BK_ERR_ARG;
    if (F == 6) return bk5col_q<Q, EB0, 6, BK_LAYOUT_TU, NB>(D, E, u, G, mass, lambda, v, s);
    if (F == 9) return bk5col_q<Q, EB0, 9, BK_LAYOUT_TU, NB>(D, E, u, G, mass, lambda, v, s);
    return BK_ERR_PREC;
}
#endif  // BK_OP_TU == 6

#if BK_OP_TU == 1
template <int Q, int EB>
int bk1_q(const double* B, long long E, const void* jxw, const void* u, void* v, int jxw_t, cudaStream_t s)
{
    using Cfg = BK1Cfg<Eng, Q, EB>;
    using S = typename Eng::S;
    static_assert(Cfg::SMEM <= 232448, "BK1 block exceeds the shared memory of an SM");
    P13<typename Eng::C, Q> prm;
    for (int i = 0; i < (Q - 1) * Q; ++i) prm.B[i] = Eng::coef(B[i]);
    for (int i = 0; i < Q * Q; ++i) prm.D[i] = Eng::coef(0.0);
    // the even-odd interpolation when B is centro-symmetric (GLL nodes,
    // Gauss points)
    const bool eo = make_eor<typename Eng::C, Q, Q - 1>(B, Q, true, +1, prm.bi, &Eng::coef) &&
                    make_eor<typename Eng::C, Q - 1, Q>(B, Q, false, +1, prm.bb, &Eng::coef);
    auto kern = eo ? bk1_kernel<Eng, Q, EB, true> : bk1_kernel<Eng, Q, EB, false>;
    const int occ = eo ? prepare<EoTag<Cfg, true>>(kern, Cfg::SMEM, Cfg::NT) : prepare<Cfg>(kern, Cfg::SMEM, Cfg::NT);
    if (occ <= 0) return BK_ERR_CUDA;
    const int grid = grid_for((E + EB - 1) / EB, occ);
    kern<<<grid, Cfg::NT, Cfg::SMEM, s>>>(prm, E, static_cast<const S*>(u), static_cast<const S*>(jxw), jxw_t,
                                          static_cast<S*>(v), dev_ctx());
    return cudaGetLastError() == cudaSuccess ? BK_OK : BK_ERR_CUDA;
}

#endif  // BK_OP_TU == 1

#if BK_OP_TU == 3
template <int Q, int EB, bool EO, int DPAR, class GS = typename Eng::S>
int bk3_launch(const P13<typename Eng::C, Q>& prm, long long E, const void* G, const void* k, const void* u, void* v,
               cudaStream_t s)
{
    using Cfg = BK3Cfg<Eng, Q, EB, DPAR>;
    using S = typename Eng::S;
    static_assert(Cfg::SMEM <= 232448, "BK3 block exceeds the shared memory of an SM");
    auto kern = bk3_kernel<Eng, Q, EB, EO, DPAR, GS>;
    const int occ = prepare<EoTag<Cfg, EO>>(kern, Cfg::SMEM, Cfg::NT);
    if (occ <= 0) return BK_ERR_CUDA;
    const int grid = grid_for((E + EB - 1) / EB, occ);
    kern<<<grid, Cfg::NT, Cfg::SMEM, s>>>(prm, E, static_cast<const S*>(u), static_cast<const GS*>(G),
                                          static_cast<const S*>(k), static_cast<S*>(v), dev_ctx());
    return cudaGetLastError() == cudaSuccess ? BK_OK : BK_ERR_CUDA;
}

// direction-parallel gradient stages for the float-float engine at q = 6..9,
// measured 8-94 % faster on GB300 (q = 8: 13.1 against 10.3 GDoF/s), with
// their own elements per block
constexpr bool sweep_dpar3(int q) { return eng_is_ff() && q >= 6 && q <= 9; }
constexpr int sweep_eb3_dpar(int q) { return q == 8 ? 2 : 3; }

template <int Q, int EB>
int bk3_q(const double* B, const double* D, long long E, const void* G, const void* k, const void* u, void* v,
          int gform, cudaStream_t s)
{
    P13<typename Eng::C, Q> prm;
    for (int i = 0; i < (Q - 1) * Q; ++i) prm.B[i] = Eng::coef(B[i]);
    for (int i = 0; i < Q * Q; ++i) prm.D[i] = Eng::coef(D[i]);
    // the even-odd contractions when B is centro-symmetric and D
    // centro-antisymmetric (GLL nodes, Gauss points)
    const bool eo = make_p13_eo<typename Eng::C, Q>(prm, B, D, &Eng::coef);
    if (eo) {
        constexpr int DP = sweep_dpar3(Q) ? 2 : 0;
        if (gform == BK_G_FF) {
            // G split ahead of time: the float-float engine's even-odd path
            if constexpr (eng_is_ff())
                return bk3_launch<Q, DP ? sweep_eb3_dpar(Q) : EB, true, DP, ff2>(prm, E, G, k, u, v, s);
            return BK_ERR_PREC;
        }
        return bk3_launch<Q, DP ? sweep_eb3_dpar(Q) : EB, true, DP>(prm, E, G, k, u, v, s);
    }
    if (gform != BK_G_STORAGE) return BK_ERR_PREC;   // split G: even-odd B and D (GLL nodes, Gauss points)
    return bk3_launch<Q, EB, false, 0>(prm, E, G, k, u, v, s);
}

#endif  // BK_OP_TU == 3

#if BK_OP_TU == 7
template <int Q, int EB, bool EO, int DPAR, class GS = typename Eng::S>
int bk3adj_launch(const P13<typename Eng::C, Q>& prm, long long E, const void* G, const void* k, const void* u,
                  const void* res, void* dk, void* dG, cudaStream_t s)
{
    using Cfg = BK3AdjCfg<Eng, Q, EB, DPAR>;
    using S = typename Eng::S;
    static_assert(Cfg::SMEM <= 232448, "BK3 adjoint block exceeds the shared memory of an SM");
    auto kern = bk3_adjoint_kernel<Eng, Q, EB, EO, DPAR, GS>;
    const int occ = prepare<EoTag<Cfg, EO>>(kern, Cfg::SMEM, Cfg::NT);
    if (occ <= 0) return BK_ERR_CUDA;
    const int grid = grid_for((E + EB - 1) / EB, occ);
    kern<<<grid, Cfg::NT, Cfg::SMEM, s>>>(prm, E, static_cast<const S*>(u), static_cast<const S*>(res),
                                          static_cast<const GS*>(G), static_cast<const S*>(k), static_cast<S*>(dk),
                                          static_cast<S*>(dG), dev_ctx());
    return cudaGetLastError() == cudaSuccess ? BK_OK : BK_ERR_CUDA;
}

// the direction-parallel gradient sweeps for the float-float engine
constexpr bool adj_dpar(int q) { return eng_is_ff() && q >= 6 && q <= 9; }
constexpr int adj_eb_dpar(int q) { return q <= 6 ? 2 : 1; }

template <int Q>
int bk3adj_q(const double* B, const double* D, long long E, const void* G, const void* k, const void* u,
             const void* res, void* dk, void* dG, int gform, cudaStream_t s)
{
    constexpr int EB = default_eb(Q) / 2 > 0 ? default_eb(Q) / 2 : 1;
    P13<typename Eng::C, Q> prm;
    for (int i = 0; i < (Q - 1) * Q; ++i) prm.B[i] = Eng::coef(B[i]);
    for (int i = 0; i < Q * Q; ++i) prm.D[i] = Eng::coef(D[i]);
    if (make_p13_eo<typename Eng::C, Q>(prm, B, D, &Eng::coef)) {
        constexpr int DP = adj_dpar(Q) ? 2 : 0;
        if (gform == BK_G_FF) {
            // G split ahead of time: the float-float engine's even-odd path
            if constexpr (eng_is_ff())
                return bk3adj_launch<Q, DP ? adj_eb_dpar(Q) : EB, true, DP, ff2>(prm, E, G, k, u, res, dk, dG, s);
            return BK_ERR_PREC;
        }
        return bk3adj_launch<Q, DP ? adj_eb_dpar(Q) : EB, true, DP>(prm, E, G, k, u, res, dk, dG, s);
    }
    if (gform != BK_G_STORAGE) return BK_ERR_PREC;
    return bk3adj_launch<Q, EB, false, 0>(prm, E, G, k, u, res, dk, dG, s);
}
#endif  // BK_OP_TU == 7

}  // namespace BK_TU_NS
using namespace BK_TU_NS;

#if BK_OP_TU == 5
#define BK_CATS_(a, b, c) a##_##b##_L##c
#define BK_CATS(a, b, c) BK_CATS_(a, b, c)
int BK_CATS(bk5_sweep, BK_SFX, BK_LAYOUT_TU)(int p, int F, const double* D, long long E, const void* u,
                                              const void* G, const void* mass, double lambda, void* v, int gform,
                                              cudaStream_t s)
{
    switch (p + 1) {
        case 2: return bk5_sweep_q<2>(F, D, E, u, G, mass, lambda, v, gform, s);
        case 3: return bk5_sweep_q<3>(F, D, E, u, G, mass, lambda, v, gform, s);
        case 4: return bk5_sweep_q<4>(F, D, E, u, G, mass, lambda, v, gform, s);
        case 5: return bk5_sweep_q<5>(F, D, E, u, G, mass, lambda, v, gform, s);
        case 6: return bk5_sweep_q<6>(F, D, E, u, G, mass, lambda, v, gform, s);
        case 7: return bk5_sweep_q<7>(F, D, E, u, G, mass, lambda, v, gform, s);
        case 8: return bk5_sweep_q<8>(F, D, E, u, G, mass, lambda, v, gform, s);
        case 9: return bk5_sweep_q<9>(F, D, E, u, G, mass, lambda, v, gform, s);
        default: return BK_ERR_ORDER;
    }
}
#endif

#if BK_OP_TU == 6
#define BK_CAT3_(a, b, c) a##_##b##_L##c
#define BK_CAT3(a, b, c) BK_CAT3_(a, b, c)
int BK_CAT3(bk5_col, BK_SFX, BK_LAYOUT_TU)(int p, int F, int eb, const double* D, long long E, const void* u,
                                            const void* G, const void* mass, double lambda, void* v, cudaStream_t s)
{
    switch (p + 1) {
        case 2: return bk5col_f<2>(F, eb, D, E, u, G, mass, lambda, v, s);
        case 3: return bk5col_f<3>(F, eb, D, E, u, G, mass, lambda, v, s);
        case 4: return bk5col_f<4>(F, eb, D, E, u, G, mass, lambda, v, s);
        case 5: return bk5col_f<5>(F, eb, D, E, u, G, mass, lambda, v, s);
        case 6: return bk5col_f<6>(F, eb, D, E, u, G, mass, lambda, v, s);
        case 7: return bk5col_f<7>(F, eb, D, E, u, G, mass, lambda, v, s);
        case 8: return bk5col_f<8>(F, eb, D, E, u, G, mass, lambda, v, s);
        case 9: return bk5col_f<9>(F, eb, D, E, u, G, mass, lambda, v, s);
        default: return BK_ERR_ORDER;
    }
}
#endif

#if BK_OP_TU == 1
// Elements per BK1 block: the default (about 128 lines) except the
// FP32-storage forms at q = 5 (BK1 p=3), whose EB = 5 (125 lines in 128
// threads) measured fastest of EB = 1..10 on GB300: FP32 88.8 against 85.0
// GDoF/s at E = 4096, 181.0 against 171.8 at E = 131072; the float-float
// engine keeps EB = 6 (35.8 against 35.1, 52.1 against 50.4).
constexpr int bk1_eb(int q) { return (q == 5 && !eng_is_ff() && !eng_is_dfma()) ? 5 : default_eb(q); }

int BK_CAT(launch_bk1, BK_SFX)(int p, long long E, const double* B, const void* jxw, const void* u, void* v,
                                int eb, int jxw_t, cudaStream_t s)
{
    (void)eb;
    switch (p + 2) {
        case 3: return bk1_q<3, default_eb(3)>(B, E, jxw, u, v, jxw_t, s);
        case 4: return bk1_q<4, default_eb(4)>(B, E, jxw, u, v, jxw_t, s);
        case 5: return bk1_q<5, bk1_eb(5)>(B, E, jxw, u, v, jxw_t, s);
        case 6: return bk1_q<6, default_eb(6)>(B, E, jxw, u, v, jxw_t, s);
        case 7: return bk1_q<7, default_eb(7)>(B, E, jxw, u, v, jxw_t, s);
        case 8: return bk1_q<8, default_eb(8)>(B, E, jxw, u, v, jxw_t, s);
        case 9: return bk1_q<9, default_eb(9)>(B, E, jxw, u, v, jxw_t, s);
        case 10: return bk1_q<10, default_eb(10)>(B, E, jxw, u, v, jxw_t, s);
        default: return BK_ERR_ORDER;
    }
}

#endif

#if BK_OP_TU == 3
int BK_CAT(launch_bk3, BK_SFX)(int p, long long E, const double* B, const double* D, const void* G, const void* k,
                                const void* u, void* v, int eb, int gform, cudaStream_t s)
{
    (void)eb;
    switch (p + 2) {
        case 3: return bk3_q<3, sweep_eb3(3)>(B, D, E, G, k, u, v, gform, s);
        case 4: return bk3_q<4, sweep_eb3(4)>(B, D, E, G, k, u, v, gform, s);
        case 5: return bk3_q<5, sweep_eb3(5)>(B, D, E, G, k, u, v, gform, s);
        case 6: return bk3_q<6, sweep_eb3(6)>(B, D, E, G, k, u, v, gform, s);
        case 7: return bk3_q<7, sweep_eb3(7)>(B, D, E, G, k, u, v, gform, s);
        case 8: return bk3_q<8, sweep_eb3(8)>(B, D, E, G, k, u, v, gform, s);
        case 9: return bk3_q<9, sweep_eb3(9)>(B, D, E, G, k, u, v, gform, s);
        case 10: return bk3_q<10, sweep_eb3(10)>(B, D, E, G, k, u, v, gform, s);
        default: return BK_ERR_ORDER;
    }
}

#endif

#if BK_OP_TU == 7
#define BK_CATL_(a, b, c) a##_##b##_L##c
#define BK_CATL(a, b, c) BK_CATL_(a, b, c)
// BK5 dispatch: kernel shape and G layout
int BK_CAT(launch_bk5, BK_SFX)(int p, long long E, const double* D, const void* G, const void* u, const void* mass,
                                double lambda, void* v, int F, int layout, int eb, int kernel, int gform,
                                cudaStream_t s)
{
    if (p < 1 || p > 8) return BK_ERR_ORDER;
    if (gform != BK_G_STORAGE && kernel == BK_KERNEL_COLUMN) return BK_ERR_PREC;   // sweep kernel only
    // AUTO, as measured on GB300 (E_p = 2^(8-p) * 4096, with and without the
    // mass term): the column kernel for the FP32-storage forms at p <= 5 with
    // G in the column layout, which it reads straight from HBM; their sweeps
    // are bound by shared-memory traffic the column kernel keeps in registers
    // (mixed p = 5: 136 against 118 GDoF/s).  The sweep kernel otherwise: at
    // p >= 6 (p = 6 mixed: 122 against 110; p = 7: 147 against 117), for the
    // float-float engine at every p (34 against 25 at p = 5), and for the
    // other layouts, where the column kernel re-lays G through shared memory
    // (mixed q = 4 at 1e8 DoFs, interleaved G: 102 against 133)
    const bool auto_col = (kernel == BK_KERNEL_AUTO) && !eng_is_ff() && !eng_is_dfma() && p <= 5 && layout == 2;
    if (kernel == BK_KERNEL_SWEEP || (kernel == BK_KERNEL_AUTO && !auto_col)) {
        switch (layout) {
            case 0: return BK_CATL(bk5_sweep, BK_SFX, 0)(p, F, D, E, u, G, mass, lambda, v, gform, s);
            case 1: return BK_CATL(bk5_sweep, BK_SFX, 1)(p, F, D, E, u, G, mass, lambda, v, gform, s);
            case 2: return BK_CATL(bk5_sweep, BK_SFX, 2)(p, F, D, E, u, G, mass, lambda, v, gform, s);
            default: return BK_ERR_PREC;
        }
    }
    switch (layout) {
        case 0: return BK_CATL(bk5_col, BK_SFX, 0)(p, F, eb, D, E, u, G, mass, lambda, v, s);
        case 1: return BK_CATL(bk5_col, BK_SFX, 1)(p, F, eb, D, E, u, G, mass, lambda, v, s);
        case 2: return BK_CATL(bk5_col, BK_SFX, 2)(p, F, eb, D, E, u, G, mass, lambda, v, s);
        default: return BK_ERR_PREC;
    }
}

int BK_CAT(launch_bk3_adjoint, BK_SFX)(int p, long long E, const double* B, const double* D, const void* G,
                                        const void* k, const void* u, const void* res, void* dk, void* dG,
                                        int gform, cudaStream_t s)
{
    switch (p + 2) {
        case 3: return bk3adj_q<3>(B, D, E, G, k, u, res, dk, dG, gform, s);
        case 4: return bk3adj_q<4>(B, D, E, G, k, u, res, dk, dG, gform, s);
        case 5: return bk3adj_q<5>(B, D, E, G, k, u, res, dk, dG, gform, s);
        case 6: return bk3adj_q<6>(B, D, E, G, k, u, res, dk, dG, gform, s);
        case 7: return bk3adj_q<7>(B, D, E, G, k, u, res, dk, dG, gform, s);
        case 8: return bk3adj_q<8>(B, D, E, G, k, u, res, dk, dG, gform, s);
        case 9: return bk3adj_q<9>(B, D, E, G, k, u, res, dk, dG, gform, s);
        case 10: return bk3adj_q<10>(B, D, E, G, k, u, res, dk, dG, gform, s);
        default: return BK_ERR_ORDER;
    }
}
#endif

}  // namespace bkg
