// bk5_col.cuh -- the BK5 kernel with a column of the element per thread.
//
// Thread (e, i, j) of a block owns the k-line u(e, i, j, 0..Q-1): the element
// layout (k fastest) makes the column contiguous, the derivative along k and
// the pointwise products with G stay in registers, and the derivatives along
// i and j read whole rows of the other threads' columns from shared memory
// (vector loads of padded rows: 8 threads of a quarter-warp hit 8 distinct
// bank groups, the threads of one row share it by broadcast).  Per batch of
// elements, two block barriers: after the columns are published, and after
// the fluxes rr, rs are published.
//
// Staging: u and G of a batch arrive by 1-D TMA bulk copies (cp.async.bulk,
// mbarrier with a bounded wait) into one of NBUF stage buffers; the copies of
// batch it + NBUF are issued as soon as batch it no longer reads its stage
// (after the second barrier), so they overlap the transposed derivatives and
// the stores of batch it and the whole of the next batches.  The staged data
// are read conflict-free: u by a cooperative pass into padded columns, G in
// the column layout G(f, k, i, j) directly (consecutive threads, consecutive
// values) or, for the other layouts, through a cooperative re-layout pass.
//
// The per-batch body (bk5_col_batch) is shared with the persistent
// mixed-order kernel of bk5_multi.cuh.
#pragma once

#include "bk_kernels.cuh"

namespace bkg {

// Row stride (in values) of a padded column buffer: a multiple of 16 bytes
// whose 16-byte chunks of 8 consecutive rows fall in distinct bank groups.
constexpr int col_rs(int q, int vbytes)
{
    return (vbytes == 4) ? (((q + 3) / 4 * 4) % 8 == 0 ? (q + 3) / 4 * 4 + 4 : (q + 3) / 4 * 4)
                         : (((q + 1) / 2 * 2) % 4 == 0 ? (q + 1) / 2 * 2 + 2 : (q + 1) / 2 * 2);
}

template <class V, int N>
__device__ __forceinline__ void ld_row(const V* p, V (&x)[N])
{
    constexpr int NB = (N * int(sizeof(V)) + 15) / 16;
    union {
        float4 f4[NB];
        V v[NB * 16 / sizeof(V)];
    } t;
#pragma unroll
    for (int b = 0; b < NB; ++b) t.f4[b] = reinterpret_cast<const float4*>(p)[b];
#pragma unroll
    for (int n = 0; n < N; ++n) x[n] = t.v[n];
}

template <class V, int N>
__device__ __forceinline__ void st_row(V* p, const V (&x)[N])
{
    constexpr int NB = (N * int(sizeof(V)) + 15) / 16;
    union {
        float4 f4[NB];
        V v[NB * 16 / sizeof(V)];
    } t;
#pragma unroll
    for (int n = 0; n < N; ++n) t.v[n] = x[n];
#pragma unroll
    for (int b = 0; b < NB; ++b) reinterpret_cast<float4*>(p)[b] = t.f4[b];
}

// G is read straight from HBM (coalesced, column layout only) by the
// FP32-storage engines; the FP64 engines stage it with TMA.
template <class Eng, int LAYOUT>
constexpr bool col_gdirect() { return LAYOUT == 2 && sizeof(typename Eng::S) == 4; }

template <class Eng, int Q, int EB, int F, int NBUF, int LAYOUT = 2>
struct BK5ColCfg {
    using S = typename Eng::S;
    using V = typename Eng::V;
    static constexpr int Q2 = Q * Q;
    static constexpr int Q3 = Q * Q * Q;
    static constexpr int RS = col_rs(Q, int(sizeof(V)));
    static constexpr int NT = ((EB * Q2 + 31) / 32) * 32;
    static constexpr int U_BYTES = stage_bytes<S>(EB * Q3);
    static constexpr bool GDIR = col_gdirect<Eng, LAYOUT>();
    static constexpr int G_BYTES = GDIR ? 0 : stage_bytes<S>(EB * F * Q3);
    static constexpr int STAGE = U_BYTES + G_BYTES;
    static constexpr int COL_BYTES = EB * Q2 * RS * int(sizeof(V));   // one padded column buffer
    static constexpr int D_BYTES = ((Q2 * int(sizeof(V)) + 15) / 16) * 16;
    // layouts 0 and 1: G of the batch re-laid in column order (f, k, i, j)
    static constexpr int GT_BYTES = (LAYOUT == 2) ? 0 : ((EB * F * Q3 * int(sizeof(V)) + 15) / 16) * 16;
    static constexpr int SMEM = NBUF * STAGE + 3 * COL_BYTES + D_BYTES + GT_BYTES + 16 * NBUF;
};

// One batch of ne elements of order Q whose u (ub) and G (gb, in LAYOUT) are
// staged densely in shared memory (with GDIR, gb is the batch's G in global
// memory, column layout).  Dp: the Q x Q matrix D(i, n) in parameter
// space (compile-time indices), Ds: the same in shared memory (run-time
// indices).  UV, R0, R1: padded column buffers of at least ne * Q^2 * RS
// values; GT: the column-order G buffer (LAYOUT != 2).  vb, mb: v and the
// optional mass at the batch's first element in global memory.  after_s2()
// runs (by every thread) right after the second barrier, once the staged data
// are no longer read.
template <class Eng, int Q, int F, int LAYOUT, bool GDIR, class AfterS2>
__device__ __forceinline__ void bk5_col_batch(const typename Eng::C* __restrict__ Dp, const typename Eng::V* Ds,
                                              const typename Eng::S* ub, const typename Eng::S* gb,
                                              typename Eng::V* UV, typename Eng::V* R0, typename Eng::V* R1,
                                              typename Eng::V* GT, int ne, int tid, int nt,
                                              typename Eng::S* __restrict__ vb, const typename Eng::S* __restrict__ mb,
                                              double lambda, AfterS2 after_s2)
{
    using S = typename Eng::S;
    using V = typename Eng::V;
    using A = typename Eng::A;
    constexpr int Q2 = Q * Q, Q3 = Q * Q * Q;
    constexpr int RS = col_rs(Q, int(sizeof(V)));
    // the float-float engine keeps the n loops rolled: its fully unrolled
    // body does not fit the instruction cache
    constexpr bool kRollN = (Eng::kId == BK_ENGINE_FF);
    const int el = tid / Q2;        // element of the batch
    const int c = tid - el * Q2;    // column (i, j)
    const int i = c / Q;
    const int j = c - i * Q;
    const bool active = el < ne;
    // lambda in the working type, tested once (an FP64 compare per point
    // would queue on the FP64 pipe)
    const bool lam_scaled = (mb != nullptr) && (lambda != 1.0);
    const V lam = Eng::load(S(lambda));
    // with GDIR, the G of this thread's column, loaded from HBM before the
    // derivatives so that the loads are in flight while they are computed
    typename Eng::S gcol[GDIR ? F : 1][GDIR ? Q : 1];
    if constexpr (GDIR) {
        if (active) {
            const S* g0 = gb + el * F * Q3 + c;
#pragma unroll
            for (int f = 0; f < F; ++f)
#pragma unroll
                for (int k = 0; k < Q; ++k) gcol[f][k] = __ldcs(g0 + (f * Q + k) * Q2);
        }
    }

    // u of the batch -> padded columns (converted); consecutive threads read
    // consecutive values
    for (int x = tid; x < ne * Q3; x += nt) {
        const int e = x / Q3;
        const int r = x - e * Q3;
        const int cc = r / Q;
        UV[(e * Q2 + cc) * RS + (r - cc * Q)] = Eng::load(ub[x]);
    }
    // layouts 0 and 1: G -> column order GT(e, f, k, c); one thread per
    // (element, factor, column) row of Q values
    if constexpr (LAYOUT != 2 && !GDIR) {
        for (int y = tid; y < ne * F * Q2; y += nt) {
            const int e = y / (F * Q2);
            const int r = y - e * (F * Q2);
            const int f = r / Q2;
            const int cc = r - f * Q2;
            const S* src = gb + e * F * Q3 + ((LAYOUT == 0) ? f * Q3 + cc * Q : (cc * F + f) * Q);
            V* dst = GT + (e * F + f) * Q3 + cc;
#pragma unroll
            for (int k = 0; k < Q; ++k) dst[k * Q2] = Eng::load(src[k]);
        }
    }
    __syncthreads();   // S1: the columns of u are published
    V ucol[Q];
    if (active) ld_row<V, Q>(UV + (el * Q2 + c) * RS, ucol);
    const S* gs = gb + el * F * Q3;
    const V* gt = GT + el * F * Q3 + c;
    auto gval = [&](int f, int k) -> V {
        if constexpr (GDIR) return Eng::load(gcol[f][k]);
        else if constexpr (LAYOUT == 2) return Eng::load(gs[(f * Q + k) * Q2 + c]);
        else return gt[(f * Q + k) * Q2];
    };

    V r2[Q];
    if (active) {
        A ar[Q], as[Q];
        const V* ubase = UV + el * Q2 * RS;
#pragma unroll
        for (int k = 0; k < Q; ++k) {
            ar[k] = Eng::zero();
            as[k] = Eng::zero();
        }
#pragma unroll(kRollN ? 1 : Q)
        for (int n = 0; n < Q; ++n) {
            V row[Q];
            ld_row<V, Q>(ubase + (n * Q + j) * RS, row);   // u(n, j, :)
            const V dr = Ds[i * Q + n];
#pragma unroll
            for (int k = 0; k < Q; ++k) Eng::vmadd(ar[k], dr, row[k]);
            ld_row<V, Q>(ubase + (i * Q + n) * RS, row);   // u(i, n, :)
            const V ds = Ds[j * Q + n];
#pragma unroll
            for (int k = 0; k < Q; ++k) Eng::vmadd(as[k], ds, row[k]);
        }
        V r0[Q], r1[Q];
#pragma unroll
        for (int k = 0; k < Q; ++k) {
            A at = Eng::zero();
#pragma unroll
            for (int n = 0; n < Q; ++n) Eng::madd(at, Dp[k * Q + n], ucol[n]);
            const V qr = Eng::result(ar[k]), qs = Eng::result(as[k]), qt = Eng::result(at);
            A a0 = Eng::zero(), a1 = Eng::zero(), a2 = Eng::zero();
            if (F == 6) {
                const V g0 = gval(0, k), g1 = gval(1, k), g2 = gval(2, k);
                const V g3 = gval(3, k), g4 = gval(4, k), g5 = gval(5, k);
                Eng::vmadd(a0, g0, qr); Eng::vmadd(a0, g1, qs); Eng::vmadd(a0, g2, qt);
                Eng::vmadd(a1, g1, qr); Eng::vmadd(a1, g3, qs); Eng::vmadd(a1, g4, qt);
                Eng::vmadd(a2, g2, qr); Eng::vmadd(a2, g4, qs); Eng::vmadd(a2, g5, qt);
            } else {
                Eng::vmadd(a0, gval(0, k), qr); Eng::vmadd(a0, gval(1, k), qs); Eng::vmadd(a0, gval(2, k), qt);
                Eng::vmadd(a1, gval(3, k), qr); Eng::vmadd(a1, gval(4, k), qs); Eng::vmadd(a1, gval(5, k), qt);
                Eng::vmadd(a2, gval(6, k), qr); Eng::vmadd(a2, gval(7, k), qs); Eng::vmadd(a2, gval(8, k), qt);
            }
            r0[k] = Eng::result(a0);
            r1[k] = Eng::result(a1);
            r2[k] = Eng::result(a2);
        }
        st_row<V, Q>(R0 + (el * Q2 + c) * RS, r0);
        st_row<V, Q>(R1 + (el * Q2 + c) * RS, r1);
    }
    __syncthreads();   // S2: fluxes published; the staged data are no longer read
    after_s2();
    if (active) {
        const V* b0 = R0 + el * Q2 * RS;
        const V* b1 = R1 + el * Q2 * RS;
        A ax[Q], ay[Q];
#pragma unroll
        for (int k = 0; k < Q; ++k) {
            ax[k] = Eng::zero();
            ay[k] = Eng::zero();
        }
#pragma unroll(kRollN ? 1 : Q)
        for (int n = 0; n < Q; ++n) {
            V row[Q];
            ld_row<V, Q>(b0 + (n * Q + j) * RS, row);   // rr(n, j, :)
            const V dx = Ds[n * Q + i];
#pragma unroll
            for (int k = 0; k < Q; ++k) Eng::vmadd(ax[k], dx, row[k]);
            ld_row<V, Q>(b1 + (i * Q + n) * RS, row);   // rs(i, n, :)
            const V dy = Ds[n * Q + j];
#pragma unroll
            for (int k = 0; k < Q; ++k) Eng::vmadd(ay[k], dy, row[k]);
        }
        S* vo = vb + el * Q3 + c * Q;
        const S* mo = (mb != nullptr) ? mb + el * Q3 + c * Q : nullptr;
#pragma unroll
        for (int k = 0; k < Q; ++k) {
            A az = Eng::zero();
#pragma unroll
            for (int n = 0; n < Q; ++n) Eng::madd(az, Dp[n * Q + k], r2[n]);
            V res;
            if constexpr (HasSum3<Eng>::value) {
                res = Eng::sum3(Eng::result(az), Eng::result(ax[k]), Eng::result(ay[k]));
            } else {
                Eng::add(az, Eng::loose(ax[k]));
                Eng::add(az, Eng::loose(ay[k]));
                res = Eng::loose(az);
            }
            if (mo != nullptr) {
                // + lambda * mass * u at the point
                A am = Eng::zero();
                Eng::add(am, res);
                V m = Eng::load(mo[k]);
                if (lam_scaled) m = Eng::mul(lam, m);
                Eng::vmadd(am, m, ucol[k]);
                res = Eng::loose(am);
            }
            vo[k] = Eng::store(res);
        }
    }
}

template <class Eng, int Q, int EB, int F, int LAYOUT, int NBUF>
__global__ void __launch_bounds__(BK5ColCfg<Eng, Q, EB, F, NBUF, LAYOUT>::NT)
    bk5_col_kernel(const __grid_constant__ P5<typename Eng::C, Q> prm, const long long E,
                   const typename Eng::S* __restrict__ u, const typename Eng::S* __restrict__ G,
                   const typename Eng::S* __restrict__ mass, const double lambda,
                   typename Eng::S* __restrict__ v, const DevCtx ctx)
{
    using Cfg = BK5ColCfg<Eng, Q, EB, F, NBUF, LAYOUT>;
    using S = typename Eng::S;
    using V = typename Eng::V;
    constexpr int Q2 = Cfg::Q2, Q3 = Cfg::Q3, RS = Cfg::RS;
    extern __shared__ __align__(16) unsigned char smem[];
    unsigned char* stage0 = smem;
    V* UV = reinterpret_cast<V*>(smem + NBUF * Cfg::STAGE);
    V* R0 = UV + EB * Q2 * RS;
    V* R1 = R0 + EB * Q2 * RS;
    V* Ds = R1 + EB * Q2 * RS;
    V* GT = reinterpret_cast<V*>(reinterpret_cast<unsigned char*>(Ds) + Cfg::D_BYTES);
    uint64_t* bars = reinterpret_cast<uint64_t*>(reinterpret_cast<unsigned char*>(GT) + Cfg::GT_BYTES);
    const int tid = threadIdx.x;
    const int nt = Cfg::NT;

    for (int x = tid; x < Q2; x += nt) Ds[x] = prm.D[x];
    if (tid == 0) {
        for (int b = 0; b < NBUF; ++b) mbar_init(&bars[b], 1);
        fence_mbar_init();
    }
    __syncthreads();

    const long long nbatch = (E + EB - 1) / EB;
    const long long stride = gridDim.x;
    // stage pointers of the batches in flight (where src[0] landed); two
    // named slots rather than an array so that they stay in registers
    static_assert(NBUF == 1 || NBUF == 2, "one or two stage buffers");
    const S* us_slot0 = nullptr;
    const S* us_slot1 = nullptr;
    const S* gs_slot0 = nullptr;
    const S* gs_slot1 = nullptr;

    auto issue = [&](long long bt, int sb) {
        const long long e0 = bt * EB;
        const int ne = int((E - e0) < EB ? (E - e0) : EB);
        unsigned char* st = stage0 + sb * Cfg::STAGE;
        uint32_t tx = 0;
        if (tid == 0) fence_proxy_async();
        const S* us_ = stage_issue<S>(st, u + e0 * Q3, ne * Q3, u + E * Q3, &bars[sb], tx, tid, nt);
        const S* gs_ = Cfg::GDIR ? nullptr
                                 : stage_issue<S>(st + Cfg::U_BYTES, G + e0 * F * Q3, ne * F * Q3, G + E * F * Q3,
                                                  &bars[sb], tx, tid, nt);
        if (sb == 0) {
            us_slot0 = us_;
            gs_slot0 = gs_;
        } else {
            us_slot1 = us_;
            gs_slot1 = gs_;
        }
        if (tid == 0) mbar_arrive_expect_tx(&bars[sb], tx);
    };

    // prologue: the first NBUF batches of this block
    for (int b = 0; b < NBUF; ++b) {
        const long long bt = blockIdx.x + b * stride;
        if (bt < nbatch) issue(bt, b);
    }

    int it = 0;
    for (long long bt = blockIdx.x; bt < nbatch; bt += stride, ++it) {
        const int sb = it % NBUF;
        const uint32_t parity = uint32_t(it / NBUF) & 1u;
        const long long e0 = bt * EB;
        const int ne = int((E - e0) < EB ? (E - e0) : EB);
        if (batch_wait_failed(&bars[sb], parity, ctx, tid)) return;
        const S* ub = (sb == 0) ? us_slot0 : us_slot1;
        const S* gb = (sb == 0) ? gs_slot0 : gs_slot1;
        if constexpr (Cfg::GDIR) gb = G + e0 * F * Q3;
        bk5_col_batch<Eng, Q, F, LAYOUT, Cfg::GDIR>(prm.D, Ds, ub, gb, UV, R0, R1, GT, ne, tid, nt, v + e0 * Q3,
                                         (mass != nullptr) ? mass + e0 * Q3 : nullptr, lambda, [&]() {
                                             const long long nb = bt + NBUF * stride;
                                             if (nb < nbatch) issue(nb, sb);
                                         });
    }
}

}  // namespace bkg
