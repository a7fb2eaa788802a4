// bk_adjoint.cuh -- the backward kernel of the variable-coefficient BK3
// operator.  With the loss L = 1/2 |A(k) u - f|^2 and the residual
// res = A(k) u - f (A symmetric, so dL/du = A(k) res is the forward kernel),
//   dL/dk(x)    = g_res(x)^T G(x) g_u(x)
//   dL/dG_aa(x) = k(x) g_res,a g_u,a                       (rr, ss, tt)
//   dL/dG_ab(x) = k(x) (g_res,a g_u,b + g_res,b g_u,a)     (rs, rt, st)
// where g_w = D B w is the reference gradient of the interpolant of w at the
// quadrature point x (each stored off-diagonal factor stands for both of its
// symmetric entries).  g_u and g_res are recomputed per element from u and
// res (three interpolation and three derivative sweeps each), not stored.
// The reference has no gradient: the forward sums are those of
// openmp/bk3_sumfact.h:63-125, the products are written from the formulas.
#pragma once

#include "bk_kernels.cuh"

namespace bkg {

// DPAR != 0: the three gradient sweeps of each field run at the same time on
// three thread groups (one shared code body), with a seventh work box.
template <class Eng, int Q, int EB, int DPAR = 0>
struct BK3AdjCfg {
    using S = typename Eng::S;
    using V = typename Eng::V;
    using WB = WBox3<Q, V>;
    static constexpr int P = Q - 1;
    static constexpr int Q3 = Q * Q * Q;
    static constexpr int P3 = P * P * P;
    static constexpr int LINES = ((EB * Q * Q + 31) / 32) * 32;
    static constexpr int NT = DPAR ? 3 * LINES : (LINES < 64 ? 64 : LINES);
    static constexpr int NBOX = DPAR ? 7 : 6;
    static constexpr int U_BYTES = stage_bytes<S>(EB * P3);
    static constexpr int G_BYTES = stage_bytes<S>(EB * 6 * Q3);
    static constexpr int K_BYTES = stage_bytes<S>(EB * Q3);
    static constexpr int W_BYTES = ((NBOX * EB * WB::size * int(sizeof(V)) + 15) / 16) * 16;
    static constexpr int SMEM = 2 * U_BYTES + G_BYTES + K_BYTES + W_BYTES + 16;
};

// u (P^3, dense S) -> gradient components at the Q^3 points in (gr, gs, gt);
// tmp is a scratch box.  gt also serves as the interpolation target unless
// DPAR.  EO: the even-odd contractions of prm.bi (interpolation,
// centro-symmetric) and prm.dg (derivative, centro-antisymmetric).  DPAR:
// the three derivative sweeps at once on three thread groups of `lines`
// threads, reading the interpolant from tmp.
template <class Eng, class WB, int Q, bool EO, int DPAR = 0>
__device__ __forceinline__ void grad_at_points(const typename Eng::S* src, typename Eng::V* tmp, typename Eng::V* gr,
                                               typename Eng::V* gs, typename Eng::V* gt, int ne,
                                               const P13<typename Eng::C, Q>& prm, int tid, int nt, int lines = 0)
{
    constexpr int P = Q - 1;
    const Mat<typename Eng::C, Q, true> Bi{prm.B};   // interpolation: M(p, i) = B[i*Q + p]
    const Mat<typename Eng::C, Q, true> Dg{prm.D};   // derivative: q(p) = sum_n w(n) D(n, p)
    load_box<Eng, WB, P, P, P>(src, P * P * P, tmp, ne, tid, nt);
    __syncthreads();
    if constexpr (DPAR) {
        static_assert(EO, "direction-parallel sweeps need the even-odd form");
        sweep_eor<Eng, WB, 0, P, P, P, Q, +1>(tmp, gr, ne, prm.bi, tid, nt);   // (Q,P,P)
        __syncthreads();
        sweep_eor<Eng, WB, 1, Q, P, P, Q, +1>(gr, gs, ne, prm.bi, tid, nt);    // (Q,Q,P)
        __syncthreads();
        sweep_eor<Eng, WB, 2, Q, Q, P, Q, +1>(gs, tmp, ne, prm.bi, tid, nt);   // w at the points
        __syncthreads();
        const int grp = tid / lines;
        if (grp < 3)
            sweep_eo_dyn<Eng, WB, Q>(tmp, grp == 0 ? gr : (grp == 1 ? gs : gt), ne, prm.dg, tid - grp * lines, lines,
                                     grp);
    } else if constexpr (EO) {
        sweep_eor<Eng, WB, 0, P, P, P, Q, +1>(tmp, gr, ne, prm.bi, tid, nt);   // (Q,P,P)
        __syncthreads();
        sweep_eor<Eng, WB, 1, Q, P, P, Q, +1>(gr, tmp, ne, prm.bi, tid, nt);   // (Q,Q,P)
        __syncthreads();
        sweep_eor<Eng, WB, 2, Q, Q, P, Q, +1>(tmp, gt, ne, prm.bi, tid, nt);   // w at the points
        __syncthreads();
        sweep_eor<Eng, WB, 0, Q, Q, Q, Q, -1>(gt, gr, ne, prm.dg, tid, nt);
        sweep_eor<Eng, WB, 1, Q, Q, Q, Q, -1>(gt, gs, ne, prm.dg, tid, nt);
        __syncthreads();
        sweep_eor<Eng, WB, 2, Q, Q, Q, Q, -1>(gt, gt, ne, prm.dg, tid, nt);
    } else {
        sweep<Eng, WB, 0, P, P, P, Q>(tmp, gr, ne, Bi, tid, nt);   // (Q,P,P)
        __syncthreads();
        sweep<Eng, WB, 1, Q, P, P, Q>(gr, tmp, ne, Bi, tid, nt);   // (Q,Q,P)
        __syncthreads();
        sweep<Eng, WB, 2, Q, Q, P, Q>(tmp, gt, ne, Bi, tid, nt);   // w at the points
        __syncthreads();
        sweep<Eng, WB, 0, Q, Q, Q, Q>(gt, gr, ne, Dg, tid, nt);
        sweep<Eng, WB, 1, Q, Q, Q, Q>(gt, gs, ne, Dg, tid, nt);
        __syncthreads();
        sweep<Eng, WB, 2, Q, Q, Q, Q>(gt, gt, ne, Dg, tid, nt);
    }
    __syncthreads();
}

template <class Eng, int Q, int EB, bool EO = false, int DPAR = 0, class GS = typename Eng::S>
__global__ void __launch_bounds__(BK3AdjCfg<Eng, Q, EB, DPAR>::NT)
    bk3_adjoint_kernel(const __grid_constant__ P13<typename Eng::C, Q> prm, const long long E,
                       const typename Eng::S* __restrict__ u, const typename Eng::S* __restrict__ res,
                       const GS* __restrict__ G, const typename Eng::S* __restrict__ kq,
                       typename Eng::S* __restrict__ dk, typename Eng::S* __restrict__ dG, const DevCtx ctx)
{
    using Cfg = BK3AdjCfg<Eng, Q, EB, DPAR>;
    using S = typename Eng::S;
    static_assert(sizeof(GS) == sizeof(S), "G is staged in the footprint of the storage type");
    using V = typename Eng::V;
    using A = typename Eng::A;
    using WB = typename Cfg::WB;
    constexpr int P3 = Cfg::P3, Q3 = Cfg::Q3;
    extern __shared__ __align__(16) unsigned char smem[];
    unsigned char* ustage = smem;
    unsigned char* rstage = ustage + Cfg::U_BYTES;
    unsigned char* gstage = rstage + Cfg::U_BYTES;
    unsigned char* kstage = gstage + Cfg::G_BYTES;
    V* W = reinterpret_cast<V*>(kstage + Cfg::K_BYTES);
    V* W0 = W;
    V* W1 = W0 + EB * WB::size;
    V* W2 = W1 + EB * WB::size;
    V* W3 = W2 + EB * WB::size;
    V* W4 = W3 + EB * WB::size;
    V* W5 = W4 + EB * WB::size;
    V* W6 = DPAR ? W5 + EB * WB::size : W0;   // the third component of g_res
    uint64_t* bar = reinterpret_cast<uint64_t*>(kstage + Cfg::K_BYTES + Cfg::W_BYTES);
    const int tid = threadIdx.x;
    const int nt = Cfg::NT;

    if (tid == 0) {
        mbar_init(bar, 1);
        fence_mbar_init();
    }
    __syncthreads();
    const long long nbatch = (E + EB - 1) / EB;
    // The next batch's u and res are copied as soon as both gradients are
    // formed (thread 0 adds their bytes to the phase without arriving), its
    // G and k once the products have read the current ones (thread 0
    // arrives): the copies overlap the products and the gradients.
    const S* us = nullptr;
    const S* rs = nullptr;
    const GS* gs = nullptr;
    const S* ks = nullptr;
    auto issue_ur = [&](long long bt, bool arrive) {
        const long long e0 = bt * EB;
        const int ne = int((E - e0) < EB ? (E - e0) : EB);
        uint32_t tx = 0;
        if (tid == 0) fence_proxy_async();
        us = stage_issue<S>(ustage, u + e0 * P3, ne * P3, u + E * P3, bar, tx, tid, nt);
        rs = stage_issue<S>(rstage, res + e0 * P3, ne * P3, res + E * P3, bar, tx, tid, nt);
        if (tid == 0) {
            if (arrive)
                mbar_arrive_expect_tx(bar, tx);
            else
                mbar_expect_tx(bar, tx);
        }
    };
    auto issue_gk = [&](long long bt) {
        const long long e0 = bt * EB;
        const int ne = int((E - e0) < EB ? (E - e0) : EB);
        uint32_t tx = 0;
        if (tid == 0) fence_proxy_async();
        gs = stage_issue<GS>(gstage, G + e0 * 6 * Q3, ne * 6 * Q3, G + E * 6 * Q3, bar, tx, tid, nt);
        ks = stage_issue<S>(kstage, kq + e0 * Q3, ne * Q3, kq + E * Q3, bar, tx, tid, nt);
        if (tid == 0) mbar_arrive_expect_tx(bar, tx);
    };
    if (blockIdx.x < nbatch) {
        issue_ur(blockIdx.x, false);
        issue_gk(blockIdx.x);
    }
    uint32_t phase = 0;
    for (long long bt = blockIdx.x; bt < nbatch; bt += gridDim.x, phase ^= 1u) {
        const long long e0 = bt * EB;
        const int ne = int((E - e0) < EB ? (E - e0) : EB);
        const long long next = bt + gridDim.x;
        if (batch_wait_failed(bar, phase, ctx, tid)) return;
        // g_u -> (W1, W2, W3) with W0 as scratch; g_res -> (W4, W5, W6), W6 = W0
        // (its last use) unless DPAR
        grad_at_points<Eng, WB, Q, EO, DPAR>(us, W0, W1, W2, W3, ne, prm, tid, nt, Cfg::LINES);
        grad_at_points<Eng, WB, Q, EO, DPAR>(rs, W0, W4, W5, W6, ne, prm, tid, nt, Cfg::LINES);
        if (next < nbatch) issue_ur(next, false);   // u and res stages are free
        for (int w = tid; w < ne * Q3; w += nt) {
            const int e = w / Q3;
            const int x = w - e * Q3;
            const int i = x / (Q * Q), j = (x / Q) % Q, k = x % Q;
            const int wi = e * WB::size + WB::at(i, j, k);
            const V ur = W1[wi], us_ = W2[wi], ut = W3[wi];
            const V rr = W4[wi], rs_ = W5[wi], rt = W6[wi];
            const GS* ge = gs + e * 6 * Q3 + x;   // factor-major
            const V g0 = Eng::load(ge[0]), g1 = Eng::load(ge[Q3]), g2 = Eng::load(ge[2 * Q3]);
            const V g3 = Eng::load(ge[3 * Q3]), g4 = Eng::load(ge[4 * Q3]), g5 = Eng::load(ge[5 * Q3]);
            const V kk = Eng::load(ks[e * Q3 + x]);
            // dL/dk = sum_ab res_a G_ab u_b
            A f0 = Eng::vfirst(g0, ur), f1 = Eng::vfirst(g1, ur), f2 = Eng::vfirst(g2, ur);
            Eng::vmadd(f0, g1, us_); Eng::vmadd(f0, g2, ut);
            Eng::vmadd(f1, g3, us_); Eng::vmadd(f1, g4, ut);
            Eng::vmadd(f2, g4, us_); Eng::vmadd(f2, g5, ut);
            A d = Eng::vfirst(rr, Eng::result(f0));
            Eng::vmadd(d, rs_, Eng::result(f1));
            Eng::vmadd(d, rt, Eng::result(f2));
            const long long o = (e0 + e) * Q3 + x;
            dk[o] = Eng::store(Eng::loose(d));
            // dL/dG
            S* go = dG + (e0 + e) * 6 * Q3 + x;
            const V kr = Eng::mul(kk, rr), ks_ = Eng::mul(kk, rs_), kt = Eng::mul(kk, rt);
            auto prod = [&](V a, V b) { return Eng::loose(Eng::vfirst(a, b)); };
            auto prod2 = [&](V a, V b, V c, V dd) {
                A t = Eng::vfirst(a, b);
                Eng::vmadd(t, c, dd);
                return Eng::loose(t);
            };
            go[0] = Eng::store(prod(kr, ur));
            go[Q3] = Eng::store(prod2(kr, us_, ks_, ur));
            go[2 * Q3] = Eng::store(prod2(kr, ut, kt, ur));
            go[3 * Q3] = Eng::store(prod(ks_, us_));
            go[4 * Q3] = Eng::store(prod2(ks_, ut, kt, us_));
            go[5 * Q3] = Eng::store(prod(kt, ut));
        }
        __syncthreads();
        if (next < nbatch) issue_gk(next);
    }
}

}  // namespace bkg
