// bk5_col.cuh -- the BK5 kernel with a column of the element per thread.
//
// Thread (e, i, j) of a block owns the k-line u(e, i, j, 0..Q-1): the element
// layout (k fastest) makes the column contiguous, the derivative along k and
// the pointwise products with G stay in registers, and the derivatives along
// i and j read whole rows of the other threads' columns from shared memory
// (vector loads of padded rows: 8 threads of a quarter-warp hit 8 distinct
// bank groups, the threads of one row share it by broadcast).  Per batch of
// EB elements, two block barriers: after the columns are published, and after
// the fluxes rr, rs are published.
//
// Staging: u and G of a batch arrive by 1-D TMA bulk copies (cp.async.bulk,
// mbarrier with a bounded wait) into one of NBUF stage buffers; the copies of
// batch it + NBUF are issued as soon as batch it no longer reads its stage
// (after the second barrier), so they overlap the transposed derivatives and
// the stores of batch it and the whole of the next batches.
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

template <class Eng, int Q, int EB, int F, int NBUF>
struct BK5ColCfg {
    using S = typename Eng::S;
    using V = typename Eng::V;
    static constexpr int Q2 = Q * Q;
    static constexpr int Q3 = Q * Q * Q;
    static constexpr int RS = col_rs(Q, int(sizeof(V)));
    static constexpr int NT = ((EB * Q2 + 31) / 32) * 32;
    static constexpr int U_BYTES = stage_bytes<S>(EB * Q3);
    static constexpr int G_BYTES = stage_bytes<S>(EB * F * Q3);
    static constexpr int STAGE = U_BYTES + G_BYTES;
    static constexpr int COL_BYTES = EB * Q2 * RS * int(sizeof(V));   // one padded column buffer
    static constexpr int D_BYTES = ((Q2 * int(sizeof(V)) + 15) / 16) * 16;
    static constexpr int SMEM = NBUF * STAGE + 3 * COL_BYTES + D_BYTES + 16 * NBUF;
};

template <int Q, int F, int LAYOUT>
__device__ __forceinline__ int g5_index(int i, int j, int f, int k)
{
    if (LAYOUT == 0) return ((f * Q + i) * Q + j) * Q + k;
    if (LAYOUT == 1) return ((i * Q + j) * F + f) * Q + k;
    return ((f * Q + k) * Q + i) * Q + j;
}

template <class Eng, int Q, int EB, int F, int LAYOUT, int NBUF>
__global__ void __launch_bounds__(BK5ColCfg<Eng, Q, EB, F, NBUF>::NT)
    bk5_col_kernel(const __grid_constant__ P5<typename Eng::C, Q> prm, const long long E,
                   const typename Eng::S* __restrict__ u, const typename Eng::S* __restrict__ G,
                   const typename Eng::S* __restrict__ mass, const double lambda,
                   typename Eng::S* __restrict__ v, const DevCtx ctx)
{
    using Cfg = BK5ColCfg<Eng, Q, EB, F, NBUF>;
    using S = typename Eng::S;
    using V = typename Eng::V;
    using A = typename Eng::A;
    constexpr int Q2 = Cfg::Q2, Q3 = Cfg::Q3, RS = Cfg::RS;
    extern __shared__ __align__(16) unsigned char smem[];
    unsigned char* stage0 = smem;
    V* UV = reinterpret_cast<V*>(smem + NBUF * Cfg::STAGE);
    V* R0 = UV + EB * Q2 * RS;
    V* R1 = R0 + EB * Q2 * RS;
    V* Ds = R1 + EB * Q2 * RS;
    uint64_t* bars = reinterpret_cast<uint64_t*>(reinterpret_cast<unsigned char*>(Ds) + Cfg::D_BYTES);

    const int tid = threadIdx.x;
    const int nt = Cfg::NT;
    const int el = tid / Q2;           // element of the batch
    const int c = tid - el * Q2;       // column (i, j)
    const int i = c / Q;
    const int j = c - i * Q;

    for (int x = tid; x < Q2; x += nt) Ds[x] = prm.D[x];
    if (tid == 0) {
        for (int b = 0; b < NBUF; ++b) mbar_init(&bars[b], 1);
        fence_mbar_init();
    }
    __syncthreads();

    const long long nbatch = (E + EB - 1) / EB;
    const long long stride = gridDim.x;
    // stage pointers of the batches in flight (where src[0] landed)
    const S* us_of[NBUF];
    const S* gs_of[NBUF];

    auto issue = [&](long long bt, int sb) {
        const long long e0 = bt * EB;
        const int ne = int((E - e0) < EB ? (E - e0) : EB);
        unsigned char* st = stage0 + sb * Cfg::STAGE;
        uint32_t tx = 0;
        if (tid == 0) fence_proxy_async();
        us_of[sb] = stage_issue<S>(st, u + e0 * Q3, ne * Q3, &bars[sb], tx, tid, nt);
        gs_of[sb] = stage_issue<S>(st + Cfg::U_BYTES, G + e0 * F * Q3, ne * F * Q3, &bars[sb], tx, tid, nt);
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
        const bool active = el < ne;
        if (batch_wait_failed(&bars[sb], parity, ctx, tid)) return;

        const S* us = us_of[sb] + el * Q3;
        const S* gs = gs_of[sb] + el * F * Q3;
        V* my = UV + (el * Q2 + c) * RS;
        V ucol[Q];
        if (active) {
#pragma unroll
            for (int k = 0; k < Q; ++k) ucol[k] = Eng::load(us[c * Q + k]);
            st_row<V, Q>(my, ucol);
        }
        __syncthreads();   // S1: the columns of u are published

        A ar[Q], as[Q];
        V r2[Q];
        if (active) {
            const V* ub = UV + el * Q2 * RS;
#pragma unroll
            for (int k = 0; k < Q; ++k) {
                ar[k] = Eng::zero();
                as[k] = Eng::zero();
            }
#pragma unroll
            for (int n = 0; n < Q; ++n) {
                V row[Q];
                ld_row<V, Q>(ub + (n * Q + j) * RS, row);   // u(n, j, :)
                const V dr = Ds[i * Q + n];
#pragma unroll
                for (int k = 0; k < Q; ++k) Eng::vmadd(ar[k], dr, row[k]);
                ld_row<V, Q>(ub + (i * Q + n) * RS, row);   // u(i, n, :)
                const V ds = Ds[j * Q + n];
#pragma unroll
                for (int k = 0; k < Q; ++k) Eng::vmadd(as[k], ds, row[k]);
            }
            V r0[Q], r1[Q];
#pragma unroll
            for (int k = 0; k < Q; ++k) {
                A at = Eng::zero();
#pragma unroll
                for (int n = 0; n < Q; ++n) Eng::madd(at, prm.D[k * Q + n], ucol[n]);
                const V qr = Eng::result(ar[k]), qs = Eng::result(as[k]), qt = Eng::result(at);
                auto g = [&](int f) { return Eng::load(gs[g5_index<Q, F, LAYOUT>(i, j, f, k)]); };
                A a0 = Eng::zero(), a1 = Eng::zero(), a2 = Eng::zero();
                if (F == 6) {
                    const V g0 = g(0), g1 = g(1), g2 = g(2), g3 = g(3), g4 = g(4), g5 = g(5);
                    Eng::vmadd(a0, g0, qr); Eng::vmadd(a0, g1, qs); Eng::vmadd(a0, g2, qt);
                    Eng::vmadd(a1, g1, qr); Eng::vmadd(a1, g3, qs); Eng::vmadd(a1, g4, qt);
                    Eng::vmadd(a2, g2, qr); Eng::vmadd(a2, g4, qs); Eng::vmadd(a2, g5, qt);
                } else {
                    Eng::vmadd(a0, g(0), qr); Eng::vmadd(a0, g(1), qs); Eng::vmadd(a0, g(2), qt);
                    Eng::vmadd(a1, g(3), qr); Eng::vmadd(a1, g(4), qs); Eng::vmadd(a1, g(5), qt);
                    Eng::vmadd(a2, g(6), qr); Eng::vmadd(a2, g(7), qs); Eng::vmadd(a2, g(8), qt);
                }
                r0[k] = Eng::result(a0);
                r1[k] = Eng::result(a1);
                r2[k] = Eng::result(a2);
            }
            st_row<V, Q>(R0 + (el * Q2 + c) * RS, r0);
            st_row<V, Q>(R1 + (el * Q2 + c) * RS, r1);
        }
        __syncthreads();   // S2: fluxes published; this batch's stage is no longer read
        {
            const long long nb = bt + NBUF * stride;
            if (nb < nbatch) issue(nb, sb);
        }
        if (active) {
            const V* b0 = R0 + el * Q2 * RS;
            const V* b1 = R1 + el * Q2 * RS;
            A ax[Q], ay[Q];
#pragma unroll
            for (int k = 0; k < Q; ++k) {
                ax[k] = Eng::zero();
                ay[k] = Eng::zero();
            }
#pragma unroll
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
            S* vo = v + (e0 + el) * Q3 + c * Q;
            const S* mo = (mass != nullptr) ? mass + (e0 + el) * Q3 + c * Q : nullptr;
#pragma unroll
            for (int k = 0; k < Q; ++k) {
                A az = Eng::zero();
#pragma unroll
                for (int n = 0; n < Q; ++n) Eng::madd(az, prm.D[n * Q + k], r2[n]);
                V res;
                if constexpr (HasSum3<Eng>::value) {
                    res = Eng::sum3(Eng::result(az), Eng::result(ax[k]), Eng::result(ay[k]));
                } else {
                    Eng::add(az, Eng::result(ax[k]));
                    Eng::add(az, Eng::result(ay[k]));
                    res = Eng::result(az);
                }
                if (mo != nullptr) {
                    // + lambda * mass * u at the point
                    A am = Eng::zero();
                    Eng::add(am, res);
                    V m = Eng::load(mo[k]);
                    if (lambda != 1.0) m = Eng::mul(Eng::load(S(lambda)), m);
                    Eng::vmadd(am, m, ucol[k]);
                    res = Eng::result(am);
                }
                vo[k] = Eng::store(res);
            }
        }
    }
}

}  // namespace bkg
