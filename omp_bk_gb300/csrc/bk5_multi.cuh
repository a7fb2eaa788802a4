// bk5_multi.cuh -- one persistent launch over elements of mixed orders.
//
// The elements of each order q = p + 1 (3..9) form a segment; a segment is
// cut into tiles of eb_q elements (eb_q chosen per order by the autotuner),
// and the tiles of all segments form one work list.  Block b of the grid
// takes tiles b, b + gridDim.x, ... (the list is ordered by decreasing cost,
// so every block gets a similar mix of orders), stages each tile's u (and G
// for the FP64 engines) by TMA into one of two stage buffers, prefetching the
// block's next tile while it computes, and runs the column batch body of
// bk5_col.cuh for the tile's order.  The operator is BK5 plus lambda times the
// collocated mass (the Helmholtz operator), G in the column layout
// G(e, f, k, i, j).
//
// bk5_multi_eo_kernel is the same launch over the sweep body of
// bk_kernels.cuh (bk5_sweep_batch) in its even-odd form, for derivative
// matrices that are centro-antisymmetric (every GLL D is): half the
// multiply-adds of the column body's derivative contractions.  One stage
// buffer per block; the overlap of copies and compute comes from the blocks
// resident on each SM, as in the single-order launches.
#pragma once

#include "bk5_col.cuh"

namespace bkg {

constexpr int kMultiQmin = 3;
constexpr int kMultiQmax = 9;
constexpr int kMultiNQ = kMultiQmax - kMultiQmin + 1;

struct MultiSeg {
    int q;               // points per direction
    int eb;              // elements per tile
    long long E;         // elements of the segment
    long long uoff;      // offset (values) of the segment in u, v and mass
    long long goff;      // offset (values) of the segment in G
};

struct MultiTile {
    int seg;
    int ne;
    long long e_first;   // first element, within the segment
};

// offset of D_q in the concatenation of D_3 .. D_9
constexpr int multi_doff(int q)
{
    int o = 0;
    for (int r = kMultiQmin; r < q; ++r) o += r * r;
    return o;
}
constexpr int kMultiDTotal = multi_doff(kMultiQmax + 1);

template <class C>
struct PMulti {
    C D[kMultiDTotal];          // D_q(i, n) at multi_doff(q) + i*q + n
    MultiSeg seg[kMultiNQ];
    int nseg;
    long long n;    // values of u, v and mass over all segments
    long long ng;   // values of G over all segments
};

// G is staged by TMA here (not held in registers): the kernel carries the
// bodies of all seven orders and must fit two blocks per SM.
template <class Eng, int NT, int NBUF>
__global__ void __launch_bounds__(NT, 2)
    bk5_multi_kernel(const __grid_constant__ PMulti<typename Eng::C> prm, const MultiTile* __restrict__ tiles,
                     const int ntiles, const typename Eng::S* __restrict__ u, const typename Eng::S* __restrict__ G,
                     const typename Eng::S* __restrict__ mass, const double lambda, typename Eng::S* __restrict__ v,
                     const int stage_bytes_, const int col_bytes, const DevCtx ctx)
{
    using S = typename Eng::S;
    using V = typename Eng::V;
    constexpr bool GDIR = false;
    extern __shared__ __align__(16) unsigned char smem[];
    unsigned char* stage0 = smem;
    V* UV = reinterpret_cast<V*>(smem + NBUF * stage_bytes_);
    V* R0 = reinterpret_cast<V*>(reinterpret_cast<unsigned char*>(UV) + col_bytes);
    V* R1 = reinterpret_cast<V*>(reinterpret_cast<unsigned char*>(R0) + col_bytes);
    V* Ds = reinterpret_cast<V*>(reinterpret_cast<unsigned char*>(R1) + col_bytes);
    uint64_t* bars = reinterpret_cast<uint64_t*>(reinterpret_cast<unsigned char*>(Ds) +
                                                 ((kMultiDTotal * int(sizeof(V)) + 15) / 16) * 16);
    const int tid = threadIdx.x;

    for (int x = tid; x < kMultiDTotal; x += NT) Ds[x] = prm.D[x];
    if (tid == 0) {
        for (int b = 0; b < NBUF; ++b) mbar_init(&bars[b], 1);
        fence_mbar_init();
    }
    __syncthreads();

    const int stride = gridDim.x;
    const S* us_slot0 = nullptr;
    const S* us_slot1 = nullptr;
    const S* gs_slot0 = nullptr;
    const S* gs_slot1 = nullptr;

    auto issue = [&](int t, int sb) {
        const MultiTile tl = tiles[t];
        const MultiSeg& sg = prm.seg[tl.seg];
        const int q3 = sg.q * sg.q * sg.q;
        unsigned char* st = stage0 + sb * stage_bytes_;
        uint32_t tx = 0;
        if (tid == 0) fence_proxy_async();
        const S* us_ = stage_issue<S>(st, u + sg.uoff + tl.e_first * q3, tl.ne * q3, u + prm.n, &bars[sb], tx, tid, NT);
        const S* gs_ = nullptr;
        if constexpr (!GDIR) {
            // the G stage follows the u stage of the largest tile
            const int ub = ((tl.ne * q3 * int(sizeof(S)) + 15) / 16) * 16 + 16;
            gs_ = stage_issue<S>(st + ub, G + sg.goff + tl.e_first * 6 * q3, tl.ne * 6 * q3, G + prm.ng, &bars[sb], tx,
                                tid, NT);
        }
        if (sb == 0) {
            us_slot0 = us_;
            gs_slot0 = gs_;
        } else {
            us_slot1 = us_;
            gs_slot1 = gs_;
        }
        if (tid == 0) mbar_arrive_expect_tx(&bars[sb], tx);
    };

    for (int b = 0; b < NBUF; ++b) {
        const int t = blockIdx.x + b * stride;
        if (t < ntiles) issue(t, b);
    }
    int it = 0;
    for (int t = blockIdx.x; t < ntiles; t += stride, ++it) {
        const int sb = it % NBUF;
        const uint32_t parity = uint32_t(it / NBUF) & 1u;
        if (batch_wait_failed(&bars[sb], parity, ctx, tid)) return;
        const MultiTile tl = tiles[t];
        const MultiSeg& sg = prm.seg[tl.seg];
        const int q3 = sg.q * sg.q * sg.q;
        const S* ub = (sb == 0) ? us_slot0 : us_slot1;
        const S* gb = GDIR ? G + sg.goff + tl.e_first * 6 * q3 : ((sb == 0) ? gs_slot0 : gs_slot1);
        S* vb = v + sg.uoff + tl.e_first * q3;
        const S* mb = (mass != nullptr) ? mass + sg.uoff + tl.e_first * q3 : nullptr;
        auto after = [&]() {
            const int tn = t + NBUF * stride;
            if (tn < ntiles) issue(tn, sb);
        };
        switch (sg.q) {
#define BK_MULTI_CASE(QQ)                                                                                       \
    case QQ:                                                                                                    \
        bk5_col_batch<Eng, QQ, 6, 2, GDIR>(prm.D + multi_doff(QQ), Ds + multi_doff(QQ), ub, gb, UV, R0, R1,   \
                                           nullptr, tl.ne, tid, NT, vb, mb, lambda, after);                    \
        break;
            BK_MULTI_CASE(3)
            BK_MULTI_CASE(4)
            BK_MULTI_CASE(5)
            BK_MULTI_CASE(6)
            BK_MULTI_CASE(7)
            BK_MULTI_CASE(8)
            BK_MULTI_CASE(9)
#undef BK_MULTI_CASE
            default:
                break;
        }
    }
}

// Shared-memory sizes of a launch over the segments: one stage buffer (the
// largest tile's u, and G when staged) and one padded column buffer.
template <class Eng>
inline void multi_smem(const MultiSeg* seg, int nseg, int& stage_bytes_, int& col_bytes, int& total, int nbuf)
{
    using S = typename Eng::S;
    using V = typename Eng::V;
    constexpr bool GDIR = false;
    stage_bytes_ = 16;
    col_bytes = 16;
    for (int s = 0; s < nseg; ++s) {
        const int q = seg[s].q, eb = seg[s].eb, q3 = q * q * q;
        int st = ((eb * q3 * int(sizeof(S)) + 15) / 16) * 16 + 16;
        if (!GDIR) st += ((eb * 6 * q3 * int(sizeof(S)) + 15) / 16) * 16 + 16;
        if (st > stage_bytes_) stage_bytes_ = st;
        const int cb = eb * q * q * col_rs(q, int(sizeof(V))) * int(sizeof(V));
        if (cb > col_bytes) col_bytes = cb;
    }
    stage_bytes_ = (stage_bytes_ + 15) / 16 * 16;
    col_bytes = (col_bytes + 15) / 16 * 16;
    total = nbuf * stage_bytes_ + 3 * col_bytes + ((kMultiDTotal * int(sizeof(V)) + 15) / 16) * 16 + 16 * nbuf;
}

// ---- even-odd sweep body -------------------------------------------------------

template <class C, int Q>
struct EOPair {
    EOMat<C, Q> eo;    // D
    EOMat<C, Q> eot;   // D^T
};

template <class C>
struct EOSet : EOPair<C, 3>, EOPair<C, 4>, EOPair<C, 5>, EOPair<C, 6>, EOPair<C, 7>, EOPair<C, 8>, EOPair<C, 9> {
    template <int Q>
    __host__ __device__ const EOPair<C, Q>& at() const
    {
        return *static_cast<const EOPair<C, Q>*>(this);
    }
    template <int Q>
    EOPair<C, Q>& at()
    {
        return *static_cast<EOPair<C, Q>*>(this);
    }
};

template <class C>
struct PMultiEO {
    EOSet<C> eo;
    MultiSeg seg[kMultiNQ];
    int nseg;
    long long n;    // values of u, v and mass over all segments
    long long ng;   // values of G over all segments
};

// Host: the even-odd forms of D_q (D(i, n) = d[i*q + n]) into P; false if D_q
// is not centro-antisymmetric.
template <class C, class Conv>
inline bool multi_eo_fill(EOSet<C>& P, int q, const double* d, Conv conv)
{
    switch (q) {
#define BK_MULTI_EO_FILL(QQ) \
    case QQ: return make_eo<C, QQ>(d, false, P.template at<QQ>().eo, conv) && make_eo<C, QQ>(d, true, P.template at<QQ>().eot, conv);
        BK_MULTI_EO_FILL(3)
        BK_MULTI_EO_FILL(4)
        BK_MULTI_EO_FILL(5)
        BK_MULTI_EO_FILL(6)
        BK_MULTI_EO_FILL(7)
        BK_MULTI_EO_FILL(8)
        BK_MULTI_EO_FILL(9)
#undef BK_MULTI_EO_FILL
        default: return false;
    }
}

// Bytes of one padded work box of eb elements of order q for values of vbytes.
inline int multi_wbox_bytes(int q, int eb, int vbytes)
{
    return eb * bk5_box(q, vbytes, 2) * vbytes;   // the element stride of WBox5
}

// Shared memory of the even-odd launch: u stage (followed by the mass stage,
// of the same size), G stage (FP64 forms only), three work boxes (each the
// largest tile's), one mbarrier.
template <class Eng>
inline void multi_eo_smem(const MultiSeg* seg, int nseg, int& u_bytes, int& g_bytes, int& w_bytes, int& total)
{
    using S = typename Eng::S;
    using V = typename Eng::V;
    u_bytes = 16;
    g_bytes = 16;
    w_bytes = 16;
    for (int s = 0; s < nseg; ++s) {
        const int q = seg[s].q, eb = seg[s].eb, q3 = q * q * q;
        // FP32 storage: G is read straight from HBM (no G stage)
        const int ub = stage_bytes<S>(eb * q3), gb = (sizeof(S) == 4) ? 16 : stage_bytes<S>(eb * 6 * q3);
        const int wb = (multi_wbox_bytes(q, eb, int(sizeof(V))) + 15) / 16 * 16;
        u_bytes = ub > u_bytes ? ub : u_bytes;
        g_bytes = gb > g_bytes ? gb : g_bytes;
        w_bytes = wb > w_bytes ? wb : w_bytes;
    }
    total = 2 * u_bytes + g_bytes + 3 * w_bytes + 16;
}

// DOT: also sum u . v over the launch, one partial per block in dot_part
// (the CG's p . A p), from compensated per-thread sums.
template <class Eng, int NT, int MINB, bool DOT = false>
__global__ void __launch_bounds__(NT, MINB)
    bk5_multi_eo_kernel(const __grid_constant__ PMultiEO<typename Eng::C> prm, const MultiTile* __restrict__ tiles,
                        const int ntiles, const typename Eng::S* __restrict__ u, const typename Eng::S* __restrict__ G,
                        const typename Eng::S* __restrict__ mass, const double lambda,
                        typename Eng::S* __restrict__ v, const int u_bytes, const int g_bytes, const int w_bytes,
                        double* __restrict__ dot_part, const DevCtx ctx)
{
    using S = typename Eng::S;
    using V = typename Eng::V;
    // FP32 storage: the pointwise stage reads G straight from HBM (coalesced:
    // G's column layout walks with the points), which leaves the largest
    // stage out of shared memory and more blocks per SM; the FP64 forms stage it
    constexpr bool GD = sizeof(S) == 4;
    extern __shared__ __align__(16) unsigned char smem[];
    unsigned char* ustage = smem;
    unsigned char* mstage = smem + u_bytes;
    unsigned char* gstage = mstage + u_bytes;
    V* W0 = reinterpret_cast<V*>(gstage + g_bytes);
    V* W1 = reinterpret_cast<V*>(reinterpret_cast<unsigned char*>(W0) + w_bytes);
    V* W2 = reinterpret_cast<V*>(reinterpret_cast<unsigned char*>(W1) + w_bytes);
    uint64_t* bar = reinterpret_cast<uint64_t*>(reinterpret_cast<unsigned char*>(W2) + w_bytes);
    const int tid = threadIdx.x;
    const int nt = blockDim.x;   // the largest tile's lines, at most NT
    if (tid == 0) {
        mbar_init(bar, 1);
        fence_mbar_init();
    }
    __syncthreads();
    ffacc dacc = acc_zero();   // u . A u over the thread's points (DOT)
    // where the staged tile's u, G and mass landed
    const S* us = nullptr;
    const S* gs = nullptr;
    const S* ms = nullptr;
    // G of tile t (thread 0 adds its bytes to the phase without arriving),
    // then u and the mass diagonal (thread 0 arrives): the next tile's G is
    // copied while the current tile finishes its transposed sweeps, u and the
    // mass (read by the last pass) right after
    auto issue_g = [&](int t) {
        if constexpr (GD) return;
        const MultiTile tl = tiles[t];
        const MultiSeg& sg = prm.seg[tl.seg];
        const int q3 = sg.q * sg.q * sg.q;
        uint32_t tx = 0;
        if (tid == 0) fence_proxy_async();
        gs = stage_issue<S>(gstage, G + sg.goff + tl.e_first * 6 * q3, tl.ne * 6 * q3, G + prm.ng, bar, tx, tid, nt);
        if (tid == 0) mbar_expect_tx(bar, tx);
    };
    auto issue_um = [&](int t) {
        const MultiTile tl = tiles[t];
        const MultiSeg& sg = prm.seg[tl.seg];
        const int q3 = sg.q * sg.q * sg.q;
        uint32_t tx = 0;
        if (tid == 0) fence_proxy_async();
        us = stage_issue<S>(ustage, u + sg.uoff + tl.e_first * q3, tl.ne * q3, u + prm.n, bar, tx, tid, nt);
        ms = (mass != nullptr)
                 ? stage_issue<S>(mstage, mass + sg.uoff + tl.e_first * q3, tl.ne * q3, mass + prm.n, bar, tx, tid, nt)
                 : nullptr;
        if (tid == 0) mbar_arrive_expect_tx(bar, tx);
    };
    if (blockIdx.x < ntiles) {
        issue_g(blockIdx.x);
        issue_um(blockIdx.x);
    }
    uint32_t phase = 0;
    for (int t = blockIdx.x; t < ntiles; t += gridDim.x, phase ^= 1u) {
        if (batch_wait_failed(bar, phase, ctx, tid)) return;
        const MultiTile tl = tiles[t];
        const MultiSeg& sg = prm.seg[tl.seg];
        const int q = sg.q;
        const int q3 = q * q * q;
        const int tn = t + gridDim.x;
        S* vb = v + sg.uoff + tl.e_first * q3;
        const S* ub = us;
        const S* gb = GD ? G + sg.goff + tl.e_first * 6 * q3 : gs;
        const S* mb = ms;
        auto early = [&]() {
            if (tn < ntiles) issue_g(tn);
        };
        switch (q) {
#define BK_MULTI_EO_CASE(QQ)                                                                                    \
    case QQ:                                                                                                    \
        bk5_sweep_batch<Eng, QQ, 6, 2, true, 0, decltype(early), DOT>(                                         \
            nullptr, prm.eo.template at<QQ>().eo, prm.eo.template at<QQ>().eot, ub, gb, W0, W1, W2, nullptr,    \
            tl.ne, tid, nt, vb, mb, lambda, &dacc, early);                                                      \
        break;
            BK_MULTI_EO_CASE(3)
            BK_MULTI_EO_CASE(4)
            BK_MULTI_EO_CASE(5)
            BK_MULTI_EO_CASE(6)
            BK_MULTI_EO_CASE(7)
            BK_MULTI_EO_CASE(8)
            BK_MULTI_EO_CASE(9)
#undef BK_MULTI_EO_CASE
            default:
                break;
        }
        if (tn < ntiles) issue_um(tn);
    }
    if constexpr (DOT) {
        // block sum of the threads' partial dot products, one value per block
        // (the work boxes are free after the last tile; no static shared
        // memory, which would shrink the dynamic limit)
        double* wsum = reinterpret_cast<double*>(W0);
        double s = double(dacc.s) + double(dacc.c);
        for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
        if ((tid & 31) == 0) wsum[tid >> 5] = s;
        __syncthreads();
        if (tid == 0) {
            double b = 0.0;
            for (int w = 0; w < (nt + 31) / 32; ++w) b += wsum[w];
            dot_part[blockIdx.x] = b;
        }
    }
}

}  // namespace bkg
