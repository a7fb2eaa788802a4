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
    int block;      // threads per block (0: the largest tile's lines)
    int gstage;     // FP32 storage: G staged by TMA (1) or read from global memory (0)
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

// Stage buffers of u and the mass of the even-odd launch: two for FP32
// storage (the next tile's copies go into one while the current tile reads
// the other), one for FP64 storage (whose G stage takes the room).
template <class Eng>
constexpr int multi_eo_nbuf()
{
    return sizeof(typename Eng::S) == 4 ? 2 : 1;
}

// Shared memory of the even-odd launch: per stage buffer a u stage followed
// by the mass stage (of the same size), the G stage (FP64, and FP32 with G
// staged), three work boxes (four with direction-parallel groups; each the
// largest tile's), one mbarrier per stage buffer.
template <class Eng>
inline void multi_eo_smem(const MultiSeg* seg, int nseg, int& u_bytes, int& g_bytes, int& w_bytes, int& total,
                          int dpar = 0, bool gst = false)
{
    using S = typename Eng::S;
    using V = typename Eng::V;
    u_bytes = 16;
    g_bytes = 16;
    w_bytes = 16;
    for (int s = 0; s < nseg; ++s) {
        const int q = seg[s].q, eb = seg[s].eb, q3 = q * q * q;
        // FP32 storage: G read straight from global memory unless staged
        const int ub = stage_bytes<S>(eb * q3), gb = (sizeof(S) == 4 && !gst) ? 16 : stage_bytes<S>(eb * 6 * q3);
        const int wb = (multi_wbox_bytes(q, eb, int(sizeof(V))) + 15) / 16 * 16;
        u_bytes = ub > u_bytes ? ub : u_bytes;
        g_bytes = gb > g_bytes ? gb : g_bytes;
        w_bytes = wb > w_bytes ? wb : w_bytes;
    }
    total = multi_eo_nbuf<Eng>() * 2 * u_bytes + g_bytes + (dpar ? 4 : 3) * w_bytes + 16;
}

// DOT: also sum u . v over the launch, one partial per block in dot_part
// (the CG's p . A p), from compensated per-thread sums.  DPAR = 2: the block
// is three thread groups that run the three gradient sweeps, and then the
// three transposed ones, at the same time (one shared code body, a fourth
// work box), as the single-order float-float kernels do.  GST (FP32
// storage): G staged by TMA instead of read straight from global memory; the
// tuner picks the faster for a plan.
//
// Staging, by mode:
//   FP32, G direct:  u and mass double-buffered; right after tile t's wait
//                    (whose block barrier also ends tile t-1's last pass, so
//                    a tile needs no barrier of its own at its end) the next
//                    tile's u and mass go into the other buffer (its barrier
//                    gets the bytes and the arrival) and its G is prefetched
//                    into L2 (one bulk prefetch), so the pointwise stage's
//                    loads wait on L2 rather than HBM.
//   FP32, G staged:  the same, but the arrival on the other buffer's barrier
//                    comes with the next tile's G, issued into the single G
//                    stage after tile t's pointwise stage.
//   FP64:            one buffer; the next tile's G after the pointwise stage
//                    (bytes only), its u and mass after the last pass (the
//                    arrival), as the single-order kernels do.
template <class Eng, int NT, int MINB, bool DOT = false, int DPAR = 0, bool GST = false>
__global__ void __launch_bounds__(NT, MINB)
    bk5_multi_eo_kernel(const __grid_constant__ PMultiEO<typename Eng::C> prm, const MultiTile* __restrict__ tiles,
                        const int ntiles, const typename Eng::S* __restrict__ u, const typename Eng::S* __restrict__ G,
                        const typename Eng::S* __restrict__ mass, const double lambda,
                        typename Eng::S* __restrict__ v, const int u_bytes, const int g_bytes, const int w_bytes,
                        double* __restrict__ dot_part, const DevCtx ctx)
{
    using S = typename Eng::S;
    using V = typename Eng::V;
    constexpr int NB = multi_eo_nbuf<Eng>();
    constexpr bool GD = NB == 2 && !GST;   // FP32, G read straight from global memory
    constexpr bool GS2 = NB == 2 && GST;   // FP32, G staged
    static_assert(NB == 2 || !GST, "FP64 storage always stages G");
    extern __shared__ __align__(16) unsigned char smem[];
    // [u 0][mass 0]([u 1][mass 1]) [G] [W0][W1][W2]([W3]) [barrier per buffer]
    unsigned char* gstage = smem + NB * 2 * u_bytes;
    V* W0 = reinterpret_cast<V*>(gstage + g_bytes);
    V* W1 = reinterpret_cast<V*>(reinterpret_cast<unsigned char*>(W0) + w_bytes);
    V* W2 = reinterpret_cast<V*>(reinterpret_cast<unsigned char*>(W1) + w_bytes);
    V* W3 = DPAR ? reinterpret_cast<V*>(reinterpret_cast<unsigned char*>(W2) + w_bytes) : nullptr;
    uint64_t* bars = reinterpret_cast<uint64_t*>(reinterpret_cast<unsigned char*>(W2) + (DPAR ? 2 : 1) * w_bytes);
    const int tid = threadIdx.x;
    const int nt = blockDim.x;   // the plan's block: tiles with more lines loop
    if (tid == 0) {
        for (int b = 0; b < NB; ++b) mbar_init(&bars[b], 1);
        fence_mbar_init();
    }
    __syncthreads();
    ffacc dacc = acc_zero();   // u . A u over the thread's points (DOT)
    // The stages of a tile are found from its descriptor (stage_at), so no
    // stage pointers stay live across tiles.
    auto g_src = [&](const MultiTile& tl) {
        const MultiSeg& sg = prm.seg[tl.seg];
        return G + sg.goff + tl.e_first * 6 * sg.q * sg.q * sg.q;
    };
    auto prefetch_g = [&](int t) {
        if (tid != 0) return;
        const MultiTile tl = tiles[t];
        const int q = prm.seg[tl.seg].q;
        prefetch_l2(g_src(tl), size_t(tl.ne) * 6 * q * q * q * sizeof(S), G + prm.ng);
    };
    // G of tile t into the G stage, counted on bars[b], with the arrival
    // (FP32 staged) or bytes only (FP64: the arrival follows with u)
    auto issue_g = [&](int t, int b, bool arrive) {
        const MultiTile tl = tiles[t];
        const int q = prm.seg[tl.seg].q;
        uint32_t tx = 0;
        if (tid == 0) fence_proxy_async();
        stage_issue<S>(gstage, g_src(tl), tl.ne * 6 * q * q * q, G + prm.ng, &bars[b], tx, tid, nt);
        if (tid == 0) {
            if (arrive)
                mbar_arrive_expect_tx(&bars[b], tx);
            else
                mbar_expect_tx(&bars[b], tx);
        }
    };
    // u and the mass diagonal of tile t into stage buffer b
    auto issue_um = [&](int t, int b, bool arrive) {
        const MultiTile tl = tiles[t];
        const MultiSeg& sg = prm.seg[tl.seg];
        const int q3 = sg.q * sg.q * sg.q;
        unsigned char* ust = smem + b * 2 * u_bytes;
        uint32_t tx = 0;
        if (tid == 0) fence_proxy_async();
        stage_issue<S>(ust, u + sg.uoff + tl.e_first * q3, tl.ne * q3, u + prm.n, &bars[b], tx, tid, nt);
        if (mass != nullptr)
            stage_issue<S>(ust + u_bytes, mass + sg.uoff + tl.e_first * q3, tl.ne * q3, mass + prm.n, &bars[b], tx,
                           tid, nt);
        if (tid == 0) {
            if (arrive)
                mbar_arrive_expect_tx(&bars[b], tx);
            else
                mbar_expect_tx(&bars[b], tx);
        }
    };
    if (blockIdx.x < ntiles) {
        if constexpr (GD) {
            prefetch_g(blockIdx.x);
            issue_um(blockIdx.x, 0, true);
        } else if constexpr (GS2) {
            issue_um(blockIdx.x, 0, false);
            issue_g(blockIdx.x, 0, true);
        } else {
            issue_g(blockIdx.x, 0, false);
            issue_um(blockIdx.x, 0, true);
        }
    }
    int it = 0;
    for (int t = blockIdx.x; t < ntiles; t += gridDim.x, ++it) {
        const int b = (NB == 2) ? (it & 1) : 0;
        const uint32_t parity = (NB == 2) ? uint32_t((it >> 1) & 1) : uint32_t(it & 1);
        const int tn = t + gridDim.x;
        // nothing of the next tile is in flight yet: a failed wait just leaves
        if (batch_wait_failed(&bars[b], parity, ctx, tid)) return;
        if constexpr (NB == 2) {
            // the other buffer was last read by the previous tile, whose last
            // pass every thread finished before the wait's barrier: the next
            // tile's u and mass go there now, so that they land while this
            // tile computes
            if (tn < ntiles) {
                if constexpr (GD) prefetch_g(tn);
                issue_um(tn, b ^ 1, GD);
            }
        }
        const MultiTile tl = tiles[t];
        const MultiSeg& sg = prm.seg[tl.seg];
        const int q = sg.q;
        const int q3 = q * q * q;
        S* vb = v + sg.uoff + tl.e_first * q3;
        const unsigned char* ust = smem + b * 2 * u_bytes;
        const S* ub = stage_at<S>(ust, u + sg.uoff + tl.e_first * q3);
        const S* gb = GD ? g_src(tl) : stage_at<S>(gstage, g_src(tl));
        const S* mb = (mass != nullptr) ? stage_at<S>(ust + u_bytes, mass + sg.uoff + tl.e_first * q3) : nullptr;
        // after the pointwise stage the G stage is free for the next tile's G
        auto early = [&]() {
            if constexpr (!GD) {
                if (tn < ntiles) issue_g(tn, NB == 2 ? (b ^ 1) : 0, NB == 2);
            }
        };
        switch (q) {
#define BK_MULTI_EO_CASE(QQ)                                                                                    \
    case QQ:                                                                                                    \
        bk5_sweep_batch<Eng, QQ, 6, 2, true, DPAR, decltype(early), DOT>(                                      \
            nullptr, prm.eo.template at<QQ>().eo, prm.eo.template at<QQ>().eot, ub, gb, W0, W1, W2, W3,         \
            tl.ne, tid, nt, vb, mb, lambda, &dacc, early, NB == 1);                                             \
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
        // FP64: the single buffer is free after the tile's last pass (the
        // batch ended with a barrier); FP32 storage: the next tile's wait
        // has the barrier that separates this tile's last pass from the
        // next writes of the boxes and of this tile's buffer
        if (NB == 1 && tn < ntiles) issue_um(tn, 0, true);
    }
    if constexpr (DOT) {
        // block sum of the threads' partial dot products, one value per block
        // (the work boxes are free after the last tile; no static shared
        // memory, which would shrink the dynamic limit)
        double* wsum = reinterpret_cast<double*>(W0);
        __syncthreads();   // the last tile's last pass may still read W0
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
