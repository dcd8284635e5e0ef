// FP64 propagator construction on the GPU and conversion to the batched format.
//
// The reference (neuwon/rxd/neuron/electric.py:78-117) assembles the matrix A
// of dV/dt coefficients (four entries per parent/child edge, already scaled
// by the half step), takes P = expm(A) with scipy and drops |P_ij| < eps.
//
// Here expm(A) is evaluated by the contour integral
//     expm(A) = 1/(2 pi i) \oint e^z (zI - A)^{-1} dz
// on the parabolic contour z(t) = N (0.1309 - 0.1194 t^2 + 0.25 i t),
// t in (-pi, pi), with the N-point midpoint rule (Weideman & Trefethen,
// "Parabolic and hyperbolic contours for computing the Bromwich integral",
// Math. Comp. 76 (2007)).  A is similar to a symmetric negative semidefinite
// matrix, so its spectrum lies on the negative real axis, which the contour
// encloses; with N = 32 the error is a few 1e-15 (absolute) for any step
// size.  Conjugate symmetry halves the work to 16 poles:
//     P = (2/N) sum_{t_k > 0} Im( e^{z_k} z'_k (z_k I - A)^{-1} ).
//
// Each resolvent (z I - A)^{-1} of a tree-structured matrix is evaluated with
// the elimination that trees allow without fill-in: for every directed edge
// the Schur pivot of the branch behind it (one leaves-to-root and one
// root-to-leaves sweep per neuron and pole), after which row i of the
// resolvent is a product of edge ratios along the path from i.  Row i of P
// is then collected by a depth-first walk outward from i that keeps entries
// with |P_ij| >= tol and stops exploring a branch once |P_ij| < tol * 1e-2.
#include <algorithm>
#include <cmath>
#include <numeric>

#include "nw_internal.cuh"

namespace nw {

constexpr int kPoles = 16;            // N/2 for N = 32
constexpr int kNodes = 2 * kPoles;
constexpr int kStackDepth = 64;
constexpr int kChainDepth = 256;
constexpr double kExploreFactor = 1e-2;
constexpr int kStatusStackOverflow = 2;
constexpr int kStatusRowMismatch = 4;
constexpr int kStatusPoolFull = 8;
constexpr int kChunk = 64;            // entries per chunk of the single-walk pool
constexpr int kMaxChunks = 256;       // chunks per row (16,384 entries)

__constant__ double2 c_z[kPoles];     // contour nodes z_k
__constant__ double2 c_w[kPoles];     // weights e^{z_k} z'_k

struct cplx {
    double re, im;
    __device__ cplx() : re(0), im(0) {}
    __device__ cplx(double r, double i) : re(r), im(i) {}
};
__device__ __forceinline__ cplx operator*(cplx a, cplx b) { return cplx(a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re); }
__device__ __forceinline__ cplx operator-(cplx a, cplx b) { return cplx(a.re - b.re, a.im - b.im); }
__device__ __forceinline__ cplx operator+(cplx a, cplx b) { return cplx(a.re + b.re, a.im + b.im); }
__device__ __forceinline__ cplx scale(double s, cplx a) { return cplx(s * a.re, s * a.im); }
__device__ __forceinline__ cplx inv(cplx a) {
    // Smith's algorithm keeps the quotient accurate over a wide range of |a|.
    if (fabs(a.re) >= fabs(a.im)) {
        double r = a.im / a.re, d = a.re + a.im * r;
        return cplx(1.0 / d, -r / d);
    } else {
        double r = a.re / a.im, d = a.re * r + a.im;
        return cplx(r / d, -1.0 / d);
    }
}
__device__ __forceinline__ cplx ld(const double2* p) { double2 v = *p; return cplx(v.x, v.y); }
__device__ __forceinline__ void st(double2* p, cplx v) { *p = make_double2(v.re, v.im); }

struct BuildArgs {
    int64_t n_seg, n_neuron;
    const int64_t* neuron_start;
    const int64_t* parent;
    const int64_t* child_ptr;   // [n_seg+1]
    const int64_t* child_idx;
    const double* cap;          // F
    const double* res;          // ohm
    const double* gsum;         // sum of 1/R over the edges at each node
    double h_s;                 // half step in seconds
    // per node, per pole (index node * kPoles + pole): the 16 lanes of a warp read
    // one node's values as one contiguous 256-byte line
    double2* down;              // pivot of the branch below node c, seen from its parent
    double2* up;                // pivot of the rest of the tree, seen from c
    double2* invT;              // 1 / total pivot: diagonal of the resolvent
    double tol, explore;
    int lump;                   // fill pass: move dropped values to the nearest kept node toward the row
    int64_t* count;             // [n_seg] kept entries per row
    const int64_t* rowptr;      // fill pass
    int32_t* out_col;
    double* out_val;
    int* status;
    // Single walk: each row's entries in chunks of kChunk taken from a pool (the
    // row's first chunk, then a link per chunk), packed into the CSR afterwards.
    int32_t* pool_col;
    double* pool_val;
    int32_t* pool_first;        // [n_seg], -1: none
    int32_t* pool_next;         // [pool_chunks]
    int* pool_top;
    int pool_chunks;
};

// One thread per (neuron, pole): the two sweeps over the neuron's tree.
__global__ void edge_pivots_kernel(const BuildArgs a) {
    int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (t >= a.n_neuron * kPoles) return;
    const int64_t j = t / kPoles;
    const int k = (int)(t % kPoles);
    const int64_t b = a.neuron_start[j], e = a.neuron_start[j + 1];
    const cplx z = cplx(c_z[k].x, c_z[k].y);
    // Node-major layout: element c of pole k lives at c * kPoles + k.
    auto D = [&](int64_t c) -> double2* { return a.down + c * kPoles + k; };
    auto U = [&](int64_t c) -> double2* { return a.up + c * kPoles + k; };
    auto IT = [&](int64_t c) -> double2* { return a.invT + c * kPoles + k; };
    // M = zI - A^T: M_cc = z + h * gsum_c / C_c; M_pc * M_cp = a_pc * a_cp with
    // a_pc = h/(R_c C_p), a_cp = h/(R_c C_c) for the edge of child c.
    for (int64_t c = b; c < e; ++c) st(D(c), z + cplx(a.h_s * a.gsum[c] / a.cap[c], 0.0));
    for (int64_t c = e - 1; c >= b; --c) {
        const int64_t p = a.parent[c];
        if (p < 0) continue;
        const double r = a.res[c];
        const double prod = (a.h_s / (r * a.cap[p])) * (a.h_s / (r * a.cap[c]));
        const cplx dc = ld(D(c));
        st(D(p), ld(D(p)) - scale(prod, inv(dc)));
    }
    // Root-to-leaves: T_p (total pivot) is known before p's children.
    for (int64_t c = b; c < e; ++c) {
        const int64_t p = a.parent[c];
        if (p < 0) {
            st(IT(c), inv(ld(D(c))));
            st(U(c), cplx(0.0, 0.0));
            continue;
        }
        const double r = a.res[c];
        const double prod = (a.h_s / (r * a.cap[p])) * (a.h_s / (r * a.cap[c]));
        const cplx dc = ld(D(c));
        const cplx Tp = inv(ld(IT(p)));
        const cplx upc = Tp + scale(prod, inv(dc));
        const cplx Tc = dc - scale(prod, inv(upc));
        st(U(c), upc);
        st(IT(c), inv(Tc));
    }
    // Store the step ratios in place of the pivots:
    //   down[c] <- a_pc / down[c]  (parent -> child),  up[c] <- a_cp / up[c]  (child -> parent).
    for (int64_t c = b; c < e; ++c) {
        const int64_t p = a.parent[c];
        if (p < 0) continue;
        const double r = a.res[c];
        st(D(c), scale(a.h_s / (r * a.cap[p]), inv(ld(D(c)))));
        st(U(c), scale(a.h_s / (r * a.cap[c]), inv(ld(U(c)))));
    }
}

// One warp per row; lanes 0..15 carry one pole each.  fill = 0 counts, 1 writes
// the CSR, 2 counts and writes the row's entries into chunks of the pool (one walk
// instead of two; a full pool sets kStatusPoolFull and the host walks twice).
// Every mode runs this same code, so they take identical decisions; the fill
// pass still checks that the row's entries land exactly in [rowptr[r], rowptr[r+1]).
//
// The walk emits a row's columns in increasing order when segments are numbered
// depth-first (children after their parent, subtrees contiguous): it first
// climbs from the row's segment i towards the root while the values stay above
// the exploration threshold (keeping each ancestor's value, which comes from
// below), then walks the reached region in preorder from the top ancestor,
// children in index order.  A chain node's value is the kept one; any other
// node's is its parent's times the edge ratio.  A node is expanded when its
// value reaches the exploration threshold (the top one, if it does not, still
// leads down the chain), so the visited set is the same as a plain walk's.
__global__ void __launch_bounds__(256) propagator_rows_kernel(const BuildArgs a, const int fill) {
    // Two rows per warp: each half-warp walks one row, one lane per pole.
    static_assert(kPoles == 16, "a half-warp carries the 16 poles");
    const int lane = threadIdx.x & 15;
    const int64_t row = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 4;
    const unsigned half_mask = (threadIdx.x & 16) ? 0xffff0000u : 0x0000ffffu;
    if (row >= a.n_seg) return;
    const int k = lane;
    // Each lane carries its pole's resolvent entry already multiplied by the
    // quadrature weight e^{z_k} z'_k and 2/N (the walk only multiplies it by edge
    // ratios, so the factor can be applied once at the row's start): the entry
    // P_ij is then the sum over the poles of the imaginary parts.
    const cplx wk = scale(2.0 / kNodes, cplx(c_w[k].x, c_w[k].y));
    auto value = [&](cplx yy) -> double {
        double v = yy.im;
#pragma unroll
        for (int off = 8; off > 0; off >>= 1) v += __shfl_xor_sync(half_mask, v, off, 16);
        return __shfl_sync(half_mask, v, 0, 16);
    };
    int32_t chain[kChainDepth];
    cplx chain_y[kChainDepth];
    int32_t st_node[kStackDepth], st_cp[kStackDepth], st_tchain[kStackDepth];
    int64_t st_tslot[kStackDepth];
    cplx st_y[kStackDepth];
    // Lumping: a dropped value goes to the nearest kept node on the tree path to the
    // row's segment.  Off the chain that is an already emitted ancestor (its slot is
    // carried down the stack) or a chain position; chain positions are settled after
    // the walk, flowing down the chain to the first kept node (the row's own
    // segment is always kept).
    int64_t chain_slot[kChainDepth];
    double carry[kChainDepth];
    const bool lump = fill && a.lump;
    int64_t kept = 0;
    int64_t out = 0;                                   // the row's next slot
    const int64_t obase = fill == 1 ? a.rowptr[row] : 0;
    const int64_t cap = fill == 1 ? a.rowptr[row + 1] - obase : 0;
    // fill = 2: the row's chunks (lane 0 alone writes entries and keeps the list).
    int32_t chunks[kMaxChunks];
    int nchunks = 0;
    auto slot = [&](int64_t sl) -> int64_t {          // index into the destination, -1: none
        if (fill == 1) return sl < cap ? obase + sl : -1;
        if (fill == 2) return (sl / kChunk) < nchunks ? (int64_t)chunks[sl / kChunk] * kChunk + sl % kChunk : -1;
        return -1;
    };
    double* const dval = fill == 2 ? a.pool_val : a.out_val;
    int32_t* const dcol = fill == 2 ? a.pool_col : a.out_col;
    // Climb.
    int depth = 0;
    int64_t cur = row;
    cplx y = wk * ld(&a.invT[row * kPoles + k]);
    chain[0] = (int32_t)row;
    chain_y[0] = y;
    double v = value(y);
    while (fabs(v) >= a.explore) {
        const int64_t p = a.parent[cur];
        if (p < 0) break;
        if (depth + 1 >= kChainDepth) {
            if (lane == 0) atomicOr(a.status, kStatusStackOverflow);
            goto done;
        }
        y = ld(&a.up[cur * kPoles + k]) * y;
        cur = p;
        ++depth;
        chain[depth] = (int32_t)cur;
        chain_y[depth] = y;
        v = value(y);
    }
    if (lump)
        for (int m = 0; m <= depth; ++m) { carry[m] = 0.0; chain_slot[m] = -1; }
    {
        // Preorder from the top; st_cp = position on the chain, -1 off it.
        int sp = 0;
        st_node[0] = chain[depth]; st_cp[0] = depth; st_y[0] = chain_y[depth];
        st_tslot[0] = -1; st_tchain[0] = depth; sp = 1;
        while (sp > 0) {
            --sp;
            const int64_t u = st_node[sp];
            const int cp = st_cp[sp];
            const cplx yu = st_y[sp];
            const int64_t tslot = st_tslot[sp];
            const int tchain = st_tchain[sp];
            const double vu = value(yu);
            const bool keep = fabs(vu) >= a.tol || (a.lump && u == row);   // lumping keeps the row's own entry
            int64_t myslot = -1;
            if (keep) {
                if (fill == 2 && lane == 0 && out % kChunk == 0) {
                    const int c = nchunks < kMaxChunks ? atomicAdd(a.pool_top, 1) : a.pool_chunks;
                    if (c < a.pool_chunks) {
                        if (nchunks == 0) a.pool_first[row] = c;
                        else a.pool_next[chunks[nchunks - 1]] = c;
                        chunks[nchunks++] = c;
                    } else {
                        atomicOr(a.status, kStatusPoolFull);
                    }
                }
                if (fill && lane == 0) {
                    const int64_t d = slot(out);
                    if (d >= 0) { dcol[d] = (int32_t)u; dval[d] = vu; }
                }
                myslot = out;
                ++out;
                ++kept;
            } else if (lump) {
                if (cp >= 0) carry[cp] += vu;
                else if (tslot >= 0) {
                    if (lane == 0) {
                        const int64_t d = slot(tslot);
                        if (d >= 0) dval[d] += vu;
                    }
                }
                else carry[tchain] += vu;
            }
            if (lump && cp >= 0) chain_slot[cp] = myslot;
            // Where this node's dropped descendants go.
            const int64_t child_tslot = keep ? myslot : (cp >= 0 ? -1 : tslot);
            const int child_tchain = cp >= 0 ? cp : tchain;
            const bool expand = fabs(vu) >= a.explore;
            const int64_t chain_child = cp > 0 ? chain[cp - 1] : -1;
            if (!expand) {
                if (chain_child < 0) continue;
                if (sp >= kStackDepth) {
                    if (lane == 0) atomicOr(a.status, kStatusStackOverflow);
                    goto done;
                }
                st_node[sp] = (int32_t)chain_child; st_cp[sp] = cp - 1; st_y[sp] = chain_y[cp - 1];
                st_tslot[sp] = -1; st_tchain[sp] = cp - 1; ++sp;
                continue;
            }
            // Children pushed last-first so that they come off the stack in index order.
            for (int64_t q = a.child_ptr[u + 1] - 1; q >= a.child_ptr[u]; --q) {
                const int64_t c = a.child_idx[q];
                if (sp >= kStackDepth) {
                    if (lane == 0) atomicOr(a.status, kStatusStackOverflow);
                    goto done;
                }
                if (c == chain_child) {
                    st_node[sp] = (int32_t)c; st_cp[sp] = cp - 1; st_y[sp] = chain_y[cp - 1];
                    st_tslot[sp] = -1; st_tchain[sp] = cp - 1;
                } else {
                    st_node[sp] = (int32_t)c; st_cp[sp] = -1; st_y[sp] = ld(&a.down[c * kPoles + k]) * yu;
                    st_tslot[sp] = child_tslot; st_tchain[sp] = child_tchain;
                }
                ++sp;
            }
        }
        if (lump && lane == 0) {
            double acc = 0.0;
            for (int m = depth; m >= 0; --m) {
                acc += carry[m];
                if (chain_slot[m] >= 0) {
                    const int64_t d = slot(chain_slot[m]);
                    if (d >= 0) dval[d] += acc;
                    acc = 0.0;
                }
            }
        }
    }
done:
    if (fill != 1 && lane == 0) a.count[row] = kept;
    if (fill == 1 && lane == 0 && out != cap) atomicOr(a.status, kStatusRowMismatch);
}

// One warp per row: the row's chunks of the pool, in order, into its CSR range.
__global__ void pool_to_rows_kernel(int64_t n, const int64_t* __restrict__ count,
                                    const int32_t* __restrict__ first, const int32_t* __restrict__ next,
                                    const int32_t* __restrict__ pcol, const double* __restrict__ pval,
                                    const int64_t* __restrict__ rowptr, int32_t* __restrict__ out_col,
                                    double* __restrict__ out_val) {
    const int64_t row = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (row >= n) return;
    const int64_t cnt = count[row], dst = rowptr[row];
    int c = first[row];
    for (int64_t e = 0; e < cnt; e += kChunk) {
        for (int k = lane; k < kChunk && e + k < cnt; k += 32) {
            out_col[dst + e + k] = pcol[(int64_t)c * kChunk + k];
            out_val[dst + e + k] = pval[(int64_t)c * kChunk + k];
        }
        if (e + kChunk < cnt) c = next[c];
    }
}

// ---------------------------------------------------------------- host

static void contour_nodes(double2* z, double2* w) {
    const double N = (double)kNodes;
    int m = 0;
    for (int k = 0; k < kNodes; ++k) {
        const double th = -M_PI + (k + 0.5) * 2.0 * M_PI / N;
        if (th <= 0) continue;
        const double zr = N * (0.1309 - 0.1194 * th * th), zi = N * 0.25 * th;
        const double dr = N * (-0.2388 * th), di = N * 0.25;
        const double ez = std::exp(zr);
        const double er = ez * std::cos(zi), ei = ez * std::sin(zi);
        z[m] = make_double2(zr, zi);
        w[m] = make_double2(er * dr - ei * di, er * di + ei * dr);
        ++m;
    }
}

// expm(A h) of the tree operator with edge "resistances" d_res (child edge) and
// node "capacities" d_cap (coefficients h_s / (R C), electric.py:85-109 form),
// pruned at tol, into an FP64 CSR with global int32 columns.
int tree_propagator_build(nw_ctx* ctx, const double* d_res, const double* d_cap, double h_s, double tol, int lump,
                          DevBuf& out_rowptr, DevBuf& out_col, DevBuf& out_val, int64_t* nnz_out) {
    const int64_t n = ctx->n_seg, nn = ctx->n_neuron;
    // Children lists and edge conductance sums (host, O(n)).
    std::vector<int64_t> cptr(n + 1, 0), cidx;
    for (int64_t i = 0; i < n; ++i) if (ctx->h_parent[i] >= 0) cptr[ctx->h_parent[i] + 1]++;
    for (int64_t i = 0; i < n; ++i) cptr[i + 1] += cptr[i];
    cidx.assign(std::max<int64_t>(cptr[n], 1), 0);
    {
        std::vector<int64_t> fillp(cptr.begin(), cptr.end() - 1);
        for (int64_t i = 0; i < n; ++i) if (ctx->h_parent[i] >= 0) cidx[fillp[ctx->h_parent[i]]++] = i;
    }
    std::vector<double> res(n), gsum(n, 0.0);
    NW_CUDA(ctx, cudaMemcpy(res.data(), d_res, 8 * n, cudaMemcpyDeviceToHost));
    for (int64_t c = 0; c < n; ++c) {
        int64_t p = ctx->h_parent[c];
        if (p < 0) continue;
        gsum[c] += 1.0 / res[c];
        gsum[p] += 1.0 / res[c];
    }
    double2 z[kPoles], w[kPoles];
    contour_nodes(z, w);
    NW_CUDA(ctx, cudaMemcpyToSymbol(c_z, z, sizeof(z)));
    NW_CUDA(ctx, cudaMemcpyToSymbol(c_w, w, sizeof(w)));

    DevBuf d_cptr, d_cidx, d_gsum, d_down, d_up, d_invT, d_count;
    DevBuf d_pcol, d_pval, d_pfirst, d_pnext, d_ptop;
    auto free_pool = [&]() { dev_free(d_pcol); dev_free(d_pval); dev_free(d_pfirst); dev_free(d_pnext); dev_free(d_ptop); };
    auto cleanup = [&]() {
        dev_free(d_cptr); dev_free(d_cidx); dev_free(d_gsum); dev_free(d_down);
        dev_free(d_up); dev_free(d_invT); dev_free(d_count);
        free_pool();
    };
    // A pool buffer is optional: a failed allocation only means two walks.
    auto try_alloc = [&](DevBuf& b, size_t bytes) {
        if (cudaMalloc(&b.ptr, bytes) != cudaSuccess) {
            b.ptr = nullptr;
            cudaGetLastError();
            return false;
        }
        b.bytes = bytes;
        return true;
    };
    int rc = NW_OK;
    do {
        if ((rc = dev_alloc(ctx, d_cptr, 8 * (n + 1))) != NW_OK) break;
        if ((rc = dev_alloc(ctx, d_cidx, 8 * cidx.size())) != NW_OK) break;
        if ((rc = dev_alloc(ctx, d_gsum, 8 * n)) != NW_OK) break;
        if ((rc = dev_alloc(ctx, d_down, sizeof(double2) * kPoles * n)) != NW_OK) break;
        if ((rc = dev_alloc(ctx, d_up, sizeof(double2) * kPoles * n)) != NW_OK) break;
        if ((rc = dev_alloc(ctx, d_invT, sizeof(double2) * kPoles * n)) != NW_OK) break;
        if ((rc = dev_alloc(ctx, d_count, 8 * n)) != NW_OK) break;
        cudaMemcpyAsync(d_cptr.ptr, cptr.data(), 8 * (n + 1), cudaMemcpyHostToDevice, ctx->stream);
        cudaMemcpyAsync(d_cidx.ptr, cidx.data(), 8 * cidx.size(), cudaMemcpyHostToDevice, ctx->stream);
        cudaMemcpyAsync(d_gsum.ptr, gsum.data(), 8 * n, cudaMemcpyHostToDevice, ctx->stream);
        cudaMemsetAsync(ctx->status.ptr, 0, 4, ctx->stream);
        BuildArgs a{};
        a.n_seg = n; a.n_neuron = nn;
        a.neuron_start = ctx->neuron_start.as<int64_t>();
        a.parent = ctx->parent.as<int64_t>();
        a.child_ptr = d_cptr.as<int64_t>(); a.child_idx = d_cidx.as<int64_t>();
        a.cap = d_cap; a.res = d_res; a.gsum = d_gsum.as<double>();
        a.h_s = h_s;
        a.down = d_down.as<double2>(); a.up = d_up.as<double2>(); a.invT = d_invT.as<double2>();
        a.tol = tol; a.explore = tol * kExploreFactor;
        a.lump = lump;
        a.count = d_count.as<int64_t>();
        a.status = ctx->status.as<int>();
        {
            int64_t threads = 128, blocks = (nn * kPoles + threads - 1) / threads;
            edge_pivots_kernel<<<(unsigned)blocks, (unsigned)threads, 0, ctx->stream>>>(a);
        }
        const int64_t rows_per_block = 16;
        const int64_t rblocks = (n + rows_per_block - 1) / rows_per_block;   // 16 rows per 256-thread block
        // One walk per row into a pool of chunks, sized to a quarter of the free
        // device memory (at most 32 chunks per row); without room, or when the pool
        // fills up, a counting walk and a filling walk as before.
        bool pooled = false;
        {
            size_t free_b = 0, total_b = 0;
            if (cudaMemGetInfo(&free_b, &total_b) != cudaSuccess) { cudaGetLastError(); free_b = 0; }
            const int64_t per_chunk = (int64_t)kChunk * (4 + 8) + 4;
            int64_t chunks = (int64_t)(0.25 * (double)free_b) / per_chunk;
            chunks = std::min<int64_t>(std::min<int64_t>(chunks, 32 * n), (int64_t)INT32_MAX - 1);
            if (ctx->prop_pool_chunks > 0) chunks = std::min<int64_t>(chunks, ctx->prop_pool_chunks);
            if (ctx->prop_walk_once && chunks >= 1 && try_alloc(d_pcol, 4 * (size_t)kChunk * chunks) &&
                try_alloc(d_pval, 8 * (size_t)kChunk * chunks) && try_alloc(d_pnext, 4 * (size_t)chunks) &&
                try_alloc(d_pfirst, 4 * (size_t)n) && try_alloc(d_ptop, 16)) {
                cudaMemsetAsync(d_pfirst.ptr, 0xff, 4 * n, ctx->stream);
                cudaMemsetAsync(d_ptop.ptr, 0, 16, ctx->stream);
                a.pool_col = d_pcol.as<int32_t>(); a.pool_val = d_pval.as<double>();
                a.pool_first = d_pfirst.as<int32_t>(); a.pool_next = d_pnext.as<int32_t>();
                a.pool_top = d_ptop.as<int>(); a.pool_chunks = (int)chunks;
                pooled = true;
            } else {
                free_pool();
            }
        }
        propagator_rows_kernel<<<(unsigned)rblocks, 256, 0, ctx->stream>>>(a, pooled ? 2 : 0);
        if (cudaGetLastError() != cudaSuccess) { rc = fail(ctx, NW_ERR_CUDA, "propagator build launch failed"); break; }
        std::vector<int64_t> cnt(n);
        int st = 0;
        cudaMemcpyAsync(cnt.data(), d_count.ptr, 8 * n, cudaMemcpyDeviceToHost, ctx->stream);
        cudaMemcpyAsync(&st, ctx->status.ptr, 4, cudaMemcpyDeviceToHost, ctx->stream);
        cudaError_t e = cudaStreamSynchronize(ctx->stream);
        if (e != cudaSuccess) { rc = cuda_fail(ctx, e, "propagator build (count pass)"); break; }
        if (pooled && (st & kStatusPoolFull) && !(st & kStatusStackOverflow)) {
            pooled = false;
            free_pool();
            cudaMemsetAsync(ctx->status.ptr, 0, 4, ctx->stream);
            propagator_rows_kernel<<<(unsigned)rblocks, 256, 0, ctx->stream>>>(a, 0);
            if (cudaGetLastError() != cudaSuccess) { rc = fail(ctx, NW_ERR_CUDA, "propagator build launch failed"); break; }
            cudaMemcpyAsync(cnt.data(), d_count.ptr, 8 * n, cudaMemcpyDeviceToHost, ctx->stream);
            cudaMemcpyAsync(&st, ctx->status.ptr, 4, cudaMemcpyDeviceToHost, ctx->stream);
            e = cudaStreamSynchronize(ctx->stream);
            if (e != cudaSuccess) { rc = cuda_fail(ctx, e, "propagator build (count pass)"); break; }
        }
        ctx->prop_walks = pooled ? 1 : 2;
        if (st & kStatusStackOverflow) {
            cudaMemsetAsync(ctx->status.ptr, 0, 4, ctx->stream);
            rc = fail(ctx, NW_ERR_LIMIT, "propagator build: walk stack or ancestor chain overflow (reach too large "
                                         "for this tolerance)");
            break;
        }
        std::vector<int64_t> rowptr(n + 1, 0);
        for (int64_t i = 0; i < n; ++i) rowptr[i + 1] = rowptr[i] + cnt[i];
        const int64_t nnz = rowptr[n];
        if ((rc = dev_alloc(ctx, out_rowptr, 8 * (n + 1))) != NW_OK) break;
        if ((rc = dev_alloc(ctx, out_col, 4 * std::max<int64_t>(nnz, 1))) != NW_OK) break;
        if ((rc = dev_alloc(ctx, out_val, 8 * std::max<int64_t>(nnz, 1))) != NW_OK) break;
        cudaMemcpyAsync(out_rowptr.ptr, rowptr.data(), 8 * (n + 1), cudaMemcpyHostToDevice, ctx->stream);
        a.rowptr = out_rowptr.as<int64_t>();
        a.out_col = out_col.as<int32_t>();
        a.out_val = out_val.as<double>();
        if (pooled) {
            pool_to_rows_kernel<<<(unsigned)((n * 32 + 255) / 256), 256, 0, ctx->stream>>>(
                n, d_count.as<int64_t>(), d_pfirst.as<int32_t>(), d_pnext.as<int32_t>(), d_pcol.as<int32_t>(),
                d_pval.as<double>(), a.rowptr, a.out_col, a.out_val);
        } else {
            propagator_rows_kernel<<<(unsigned)rblocks, 256, 0, ctx->stream>>>(a, 1);
        }
        if (cudaGetLastError() != cudaSuccess) { rc = fail(ctx, NW_ERR_CUDA, "propagator build launch failed"); break; }
        cudaMemcpyAsync(&st, ctx->status.ptr, 4, cudaMemcpyDeviceToHost, ctx->stream);
        e = cudaStreamSynchronize(ctx->stream);
        if (e != cudaSuccess) { rc = cuda_fail(ctx, e, "propagator build (fill pass)"); break; }
        if (st & kStatusRowMismatch) {
            cudaMemsetAsync(ctx->status.ptr, 0, 4, ctx->stream);
            rc = fail(ctx, NW_ERR_STATE, "propagator build: count and fill passes disagree");
            break;
        }
        if (nnz_out) *nnz_out = nnz;
    } while (0);
    cleanup();
    return rc;
}

int propagator_build(nw_ctx* ctx, double tol, int64_t* nnz_out) {
    int64_t nnz = 0;
    NW_CHECK(tree_propagator_build(ctx, ctx->res64.as<double>(), ctx->cap64.as<double>(),
                                   0.5 * ctx->time_step * 1e-3, tol, ctx->prop_lump ? 1 : 0, ctx->p_rowptr, ctx->p_col,
                                   ctx->p_val, &nnz));
    ctx->nnz64 = nnz;
    if (nnz_out) *nnz_out = nnz;
    return NW_OK;
}

int propagator_from_host(nw_ctx* ctx, const int64_t* rowptr, const int64_t* col, const double* val,
                         int64_t nnz) {
    const int64_t n = ctx->n_seg;
    NW_CHECK(dev_alloc(ctx, ctx->p_rowptr, 8 * (n + 1)));
    NW_CHECK(dev_alloc(ctx, ctx->p_col, 4 * std::max<int64_t>(nnz, 1)));
    NW_CHECK(dev_alloc(ctx, ctx->p_val, 8 * std::max<int64_t>(nnz, 1)));
    std::vector<int32_t> c32(nnz);
    for (int64_t e = 0; e < nnz; ++e) c32[e] = (int32_t)col[e];
    NW_CUDA(ctx, cudaMemcpyAsync(ctx->p_rowptr.ptr, rowptr, 8 * (n + 1), cudaMemcpyHostToDevice, ctx->stream));
    if (nnz) {
        NW_CUDA(ctx, cudaMemcpyAsync(ctx->p_col.ptr, c32.data(), 4 * nnz, cudaMemcpyHostToDevice, ctx->stream));
        NW_CUDA(ctx, cudaMemcpyAsync(ctx->p_val.ptr, val, 8 * nnz, cudaMemcpyHostToDevice, ctx->stream));
    }
    NW_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    ctx->nnz64 = nnz;
    return NW_OK;
}

// ------------------------------------------------- charge-conserving pruning

// One warp per row: diag += 1 - sum(row), summed in FP64 in a fixed order.
__global__ void conserve_rows_kernel(int64_t n, const int64_t* prow, const int32_t* pcol, double* pval,
                                     int* status) {
    const int lane = threadIdx.x & 31;
    const int64_t r = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
    if (r >= n) return;
    double sum = 0.0;
    int64_t diag = -1;
    for (int64_t k = prow[r] + lane; k < prow[r + 1]; k += 32) {
        sum += pval[k];
        if (pcol[k] == (int32_t)r) diag = k;
    }
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) sum += __shfl_xor_sync(0xffffffffu, sum, off);
    const unsigned has = __ballot_sync(0xffffffffu, diag >= 0);
    if (!has) {
        if (lane == 0) atomicOr(status, 8);
        return;
    }
    if (lane == __ffs(has) - 1) pval[diag] += 1.0 - sum;
}

int csr_conserve(nw_ctx* ctx, DevBuf& rowptr, DevBuf& col, DevBuf& val) {
    const int64_t n = ctx->n_seg;
    cudaMemsetAsync(ctx->status.ptr, 0, 4, ctx->stream);
    conserve_rows_kernel<<<(unsigned)((n * 32 + 255) / 256), 256, 0, ctx->stream>>>(
        n, rowptr.as<int64_t>(), col.as<int32_t>(), val.as<double>(), ctx->status.as<int>());
    int st = 0;
    NW_CUDA(ctx, cudaMemcpyAsync(&st, ctx->status.ptr, 4, cudaMemcpyDeviceToHost, ctx->stream));
    NW_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    if (st & 8) {
        cudaMemsetAsync(ctx->status.ptr, 0, 4, ctx->stream);
        return fail(ctx, NW_ERR_STATE, "nw_propagator_conserve: a row has no diagonal entry");
    }
    return NW_OK;
}

int propagator_conserve(nw_ctx* ctx) { return csr_conserve(ctx, ctx->p_rowptr, ctx->p_col, ctx->p_val); }

// ------------------------------------------------- batched difference form

__global__ void rows_count_kernel(int64_t n, const int64_t* prow, const int32_t* pcol, int64_t* cnt) {
    int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (r >= n) return;
    int64_t c = 0;
    for (int64_t k = prow[r]; k < prow[r + 1]; ++k) c += (pcol[k] != (int32_t)r);
    cnt[r] = (c + 7) & ~(int64_t)7;   // 8-entry rows: 16-byte aligned vectors and bulk copies
}

// Off-diagonal entries of each row (warp per row, order kept) with columns
// relative to the row's neuron (u16, batched format) or global (i32, wide
// format), zero padding, and leak = 1 - row sum accumulated in FP64.
template <typename real, typename CT>
__global__ void rows_fill_kernel(int64_t n, const int64_t* neuron_of_row_base, const int64_t* prow,
                                 const int32_t* pcol, const double* pval, const int64_t* brow,
                                 CT* bcol, real* bval, real* leak) {
    const int lane = threadIdx.x & 31;
    const int64_t r = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
    if (r >= n) return;
    const int64_t base = neuron_of_row_base ? neuron_of_row_base[r] : 0;
    int64_t ob = brow[r];
    double sum = 0.0;
    for (int64_t k0 = prow[r]; k0 < prow[r + 1]; k0 += 32) {
        const int64_t k = k0 + lane;
        const bool valid = k < prow[r + 1];
        const int32_t c = valid ? pcol[k] : -1;
        const double v = valid ? pval[k] : 0.0;
        sum += v;
        const bool off = valid && c != (int32_t)r;
        const unsigned mask = __ballot_sync(0xffffffffu, off);
        const int pos = __popc(mask & ((1u << lane) - 1u));
        if (off) { bcol[ob + pos] = (CT)(c - base); bval[ob + pos] = (real)v; }
        ob += __popc(mask);
    }
    // Padding points at the row itself (x_i - x_i = 0 in the difference form).
    for (int64_t k = ob + lane; k < brow[r + 1]; k += 32) { bcol[k] = (CT)(r - base); bval[k] = real(0); }
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) sum += __shfl_xor_sync(0xffffffffu, sum, off);
    if (lane == 0) leak[r] = (real)(1.0 - sum);
}

void free_wide(nw_ctx* ctx) {
    for (DevBuf* b : {&ctx->w_rowptr, &ctx->w_col, &ctx->w_val, &ctx->w_leak}) dev_free(*b);
    ctx->w_ok = false;
    ctx->nnz_w = 0;
}

// One row format from an FP64 CSR (src_*): columns relative to the row's
// neuron (u16, batched format) or global (i32, wide format).
template <typename CT>
int csr_to_rows(nw_ctx* ctx, const DevBuf& src_row, const DevBuf& src_col, const DevBuf& src_val, bool relative,
                DevBuf& R, DevBuf& C, DevBuf& V, DevBuf& L, int64_t* nnz_out) {
    const int64_t n = ctx->n_seg;
    DevBuf d_cnt, d_base;
    NW_CHECK(dev_alloc(ctx, d_cnt, 8 * n));
    int rc = NW_OK;
    if (relative) {
        rc = dev_alloc(ctx, d_base, 8 * n);
        if (rc != NW_OK) { dev_free(d_cnt); return rc; }
        std::vector<int64_t> base(n);
        for (int64_t j = 0; j < ctx->n_neuron; ++j)
            for (int64_t i = ctx->h_neuron_start[j]; i < ctx->h_neuron_start[j + 1]; ++i) base[i] = ctx->h_neuron_start[j];
        cudaMemcpyAsync(d_base.ptr, base.data(), 8 * n, cudaMemcpyHostToDevice, ctx->stream);
        cudaStreamSynchronize(ctx->stream);
    }
    rows_count_kernel<<<(unsigned)((n + 255) / 256), 256, 0, ctx->stream>>>(
        n, src_row.as<int64_t>(), src_col.as<int32_t>(), d_cnt.as<int64_t>());
    std::vector<int64_t> cnt(n), brow(n + 1, 0);
    cudaMemcpyAsync(cnt.data(), d_cnt.ptr, 8 * n, cudaMemcpyDeviceToHost, ctx->stream);
    cudaError_t e = cudaStreamSynchronize(ctx->stream);
    if (e != cudaSuccess) { dev_free(d_cnt); dev_free(d_base); return cuda_fail(ctx, e, "row format count"); }
    for (int64_t i = 0; i < n; ++i) brow[i + 1] = brow[i] + cnt[i];
    const int64_t nb = brow[n];
    const size_t rs = (size_t)ctx->precision;
    do {
        if ((rc = dev_alloc(ctx, R, 8 * (n + 1))) != NW_OK) break;
        if ((rc = dev_alloc(ctx, C, sizeof(CT) * std::max<int64_t>(nb, 8))) != NW_OK) break;
        if ((rc = dev_alloc(ctx, V, rs * std::max<int64_t>(nb, 8))) != NW_OK) break;
        if ((rc = dev_alloc(ctx, L, rs * n)) != NW_OK) break;
        cudaMemcpyAsync(R.ptr, brow.data(), 8 * (n + 1), cudaMemcpyHostToDevice, ctx->stream);
        const unsigned blocks = (unsigned)((n * 32 + 255) / 256);
        const int64_t* base = relative ? d_base.as<int64_t>() : nullptr;
        if (ctx->precision == NW_F64)
            rows_fill_kernel<double, CT><<<blocks, 256, 0, ctx->stream>>>(
                n, base, src_row.as<int64_t>(), src_col.as<int32_t>(), src_val.as<double>(),
                R.as<int64_t>(), C.as<CT>(), V.as<double>(), L.as<double>());
        else
            rows_fill_kernel<float, CT><<<blocks, 256, 0, ctx->stream>>>(
                n, base, src_row.as<int64_t>(), src_col.as<int32_t>(), src_val.as<double>(),
                R.as<int64_t>(), C.as<CT>(), V.as<float>(), L.as<float>());
        e = cudaStreamSynchronize(ctx->stream);
        if (e != cudaSuccess) { rc = cuda_fail(ctx, e, "row format fill"); break; }
        if (nnz_out) *nnz_out = nb;
    } while (0);
    dev_free(d_cnt);
    dev_free(d_base);
    return rc;
}
template int csr_to_rows<uint16_t>(nw_ctx*, const DevBuf&, const DevBuf&, const DevBuf&, bool, DevBuf&, DevBuf&,
                                   DevBuf&, DevBuf&, int64_t*);
template int csr_to_rows<int32_t>(nw_ctx*, const DevBuf&, const DevBuf&, const DevBuf&, bool, DevBuf&, DevBuf&,
                                  DevBuf&, DevBuf&, int64_t*);

// ------------------------------------------------- pair (flux) format

// Entry (i, c) of row i belongs to row i when c_i < c_c (ties: i < c).
__device__ __forceinline__ bool pair_owner(const double* cap, int64_t i, int64_t c) {
    const double ci = cap[i], cc = cap[c];
    return ci < cc || (ci == cc && i < c);
}

__global__ void flux_count_kernel(int64_t n, const int64_t* prow, const int32_t* pcol, const double* cap,
                                  int64_t* cnt) {
    int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (r >= n) return;
    int64_t c = 0;
    for (int64_t k = prow[r]; k < prow[r + 1]; ++k) {
        const int64_t col = pcol[k];
        c += (col != r && pair_owner(cap, r, col)) ? 1 : 0;
    }
    cnt[r] = (c + 3) & ~(int64_t)3;   // 4-entry vectors
}

template <typename real>
__global__ void flux_fill_kernel(int64_t n, const int64_t* row_base, const double* row_cmax, const int64_t* prow,
                                 const int32_t* pcol, const double* pval, const double* cap, const int64_t* frow,
                                 uint16_t* fcol, real* fval, real* leak, real* rc) {
    const int lane = threadIdx.x & 31;
    const int64_t r = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
    if (r >= n) return;
    const int64_t base = row_base[r];
    const double cmax = row_cmax[r];
    const double scale = cap[r] / cmax;
    int64_t ob = frow[r];
    double sum = 0.0;
    for (int64_t k0 = prow[r]; k0 < prow[r + 1]; k0 += 32) {
        const int64_t k = k0 + lane;
        const bool valid = k < prow[r + 1];
        const int32_t c = valid ? pcol[k] : -1;
        const double v = valid ? pval[k] : 0.0;
        sum += v;
        const bool own = valid && c != (int32_t)r && pair_owner(cap, r, c);
        const unsigned mask = __ballot_sync(0xffffffffu, own);
        const int pos = __popc(mask & ((1u << lane) - 1u));
        if (own) { fcol[ob + pos] = (uint16_t)(c - base); fval[ob + pos] = (real)(v * scale); }
        ob += __popc(mask);
    }
    for (int64_t k = ob + lane; k < frow[r + 1]; k += 32) { fcol[k] = (uint16_t)(r - base); fval[k] = real(0); }
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) sum += __shfl_xor_sync(0xffffffffu, sum, off);
    // c_max / c_r times the fixed-point scale of the pair sums.
    const double fixed = sizeof(real) == 4 ? kPairScaleF32 : kPairScaleF64;
    if (lane == 0) { leak[r] = (real)(1.0 - sum); rc[r] = (real)(cmax / cap[r] * fixed); }
}

void free_flux(nw_ctx* ctx) {
    for (DevBuf* b : {&ctx->f_rowptr, &ctx->f_col, &ctx->f_val, &ctx->f_leak, &ctx->f_rc, &ctx->f_acc}) dev_free(*b);
    ctx->f_ok = false;
    ctx->nnz_f = 0;
}

int ensure_flux(nw_ctx* ctx) {
    if (ctx->f_ok) return NW_OK;
    if (ctx->max_neuron > 65535) return fail(ctx, NW_ERR_LIMIT, "pair format: a neuron has more than 65,535 segments");
    const int64_t n = ctx->n_seg;
    std::vector<double> cap(n);
    NW_CUDA(ctx, cudaMemcpy(cap.data(), ctx->cap64.ptr, 8 * n, cudaMemcpyDeviceToHost));
    std::vector<int64_t> base(n);
    std::vector<double> cmax(n);
    for (int64_t j = 0; j < ctx->n_neuron; ++j) {
        double m = 0.0;
        for (int64_t i = ctx->h_neuron_start[j]; i < ctx->h_neuron_start[j + 1]; ++i) m = std::max(m, cap[i]);
        for (int64_t i = ctx->h_neuron_start[j]; i < ctx->h_neuron_start[j + 1]; ++i) { base[i] = ctx->h_neuron_start[j]; cmax[i] = m; }
    }
    DevBuf d_cnt, d_base, d_cmax;
    auto cleanup = [&]() { dev_free(d_cnt); dev_free(d_base); dev_free(d_cmax); };
    int rc = NW_OK;
    do {
        if ((rc = dev_alloc(ctx, d_cnt, 8 * n)) != NW_OK) break;
        if ((rc = dev_alloc(ctx, d_base, 8 * n)) != NW_OK) break;
        if ((rc = dev_alloc(ctx, d_cmax, 8 * n)) != NW_OK) break;
        cudaMemcpyAsync(d_base.ptr, base.data(), 8 * n, cudaMemcpyHostToDevice, ctx->stream);
        cudaMemcpyAsync(d_cmax.ptr, cmax.data(), 8 * n, cudaMemcpyHostToDevice, ctx->stream);
        flux_count_kernel<<<(unsigned)((n + 255) / 256), 256, 0, ctx->stream>>>(
            n, ctx->p_rowptr.as<int64_t>(), ctx->p_col.as<int32_t>(), ctx->cap64.as<double>(), d_cnt.as<int64_t>());
        std::vector<int64_t> cnt(n), frow(n + 1, 0);
        cudaMemcpyAsync(cnt.data(), d_cnt.ptr, 8 * n, cudaMemcpyDeviceToHost, ctx->stream);
        cudaError_t e = cudaStreamSynchronize(ctx->stream);
        if (e != cudaSuccess) { rc = cuda_fail(ctx, e, "pair format count"); break; }
        for (int64_t i = 0; i < n; ++i) frow[i + 1] = frow[i] + cnt[i];
        const int64_t nf = frow[n];
        const size_t rs = (size_t)ctx->precision;
        if ((rc = dev_alloc(ctx, ctx->f_rowptr, 8 * (n + 1))) != NW_OK) break;
        if ((rc = dev_alloc(ctx, ctx->f_col, 2 * std::max<int64_t>(nf, 8))) != NW_OK) break;
        if ((rc = dev_alloc(ctx, ctx->f_val, rs * std::max<int64_t>(nf, 8))) != NW_OK) break;
        if ((rc = dev_alloc(ctx, ctx->f_leak, rs * n)) != NW_OK) break;
        if ((rc = dev_alloc(ctx, ctx->f_rc, rs * n)) != NW_OK) break;
        if ((rc = dev_alloc(ctx, ctx->f_acc, 8 * n)) != NW_OK) break;
        cudaMemcpyAsync(ctx->f_rowptr.ptr, frow.data(), 8 * (n + 1), cudaMemcpyHostToDevice, ctx->stream);
        cudaMemsetAsync(ctx->f_acc.ptr, 0, 8 * n, ctx->stream);
        const unsigned blocks = (unsigned)((n * 32 + 255) / 256);
        if (ctx->precision == NW_F64)
            flux_fill_kernel<double><<<blocks, 256, 0, ctx->stream>>>(
                n, d_base.as<int64_t>(), d_cmax.as<double>(), ctx->p_rowptr.as<int64_t>(), ctx->p_col.as<int32_t>(),
                ctx->p_val.as<double>(), ctx->cap64.as<double>(), ctx->f_rowptr.as<int64_t>(),
                ctx->f_col.as<uint16_t>(), ctx->f_val.as<double>(), ctx->f_leak.as<double>(), ctx->f_rc.as<double>());
        else
            flux_fill_kernel<float><<<blocks, 256, 0, ctx->stream>>>(
                n, d_base.as<int64_t>(), d_cmax.as<double>(), ctx->p_rowptr.as<int64_t>(), ctx->p_col.as<int32_t>(),
                ctx->p_val.as<double>(), ctx->cap64.as<double>(), ctx->f_rowptr.as<int64_t>(),
                ctx->f_col.as<uint16_t>(), ctx->f_val.as<float>(), ctx->f_leak.as<float>(), ctx->f_rc.as<float>());
        e = cudaStreamSynchronize(ctx->stream);
        if (e != cudaSuccess) { rc = cuda_fail(ctx, e, "pair format fill"); break; }
        ctx->nnz_f = nf;
        ctx->f_ok = true;
    } while (0);
    cleanup();
    return rc;
}

// ------------------------------------------------- quad format

// Quads of row r: windows [b, b+3] (b <= neuron end - 4, and b = the neuron's first
// segment for neurons of fewer than 4) opened at an entry that does not fit the
// current window, in the row's entry order.  With columns in
// increasing order every window is as full as the runs allow.
__device__ __forceinline__ int64_t quad_window(int64_t c, int64_t lo, int64_t hi) {
    int64_t b = c;
    if (b > hi - 4) b = hi - 4;
    if (b < lo) b = lo;
    return b;
}

__global__ void quad_count_kernel(int64_t n, const int64_t* nstart_of_row, const int64_t* nend_of_row,
                                  const int64_t* prow, const int32_t* pcol, int64_t* cnt) {
    const int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (r >= n) return;
    const int64_t lo = nstart_of_row[r], hi = nend_of_row[r];
    int64_t q = 0, b = -1, last = -1;
    for (int64_t k = prow[r]; k < prow[r + 1]; ++k) {
        const int64_t c = pcol[k];
        if (c == r) continue;
        if (b < 0 || c < b || c > b + 3 || c <= last) { b = quad_window(c, lo, hi); ++q; }
        last = c;
    }
    cnt[r] = q;
}

template <typename real, typename BT>
__global__ void quad_fill_kernel(int64_t n, const int64_t* nstart_of_row, const int64_t* nend_of_row,
                                 const int64_t* prow, const int32_t* pcol, const double* pval,
                                 const int64_t* qrow, BT* qbase, real* qval, int relative) {
    const int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (r >= n) return;
    const int64_t lo = nstart_of_row[r], hi = nend_of_row[r];
    int64_t q = qrow[r] - 1, b = -1, last = -1;
    for (int64_t k = prow[r]; k < prow[r + 1]; ++k) {
        const int64_t c = pcol[k];
        if (c == r) continue;
        if (b < 0 || c < b || c > b + 3 || c <= last) {
            b = quad_window(c, lo, hi);
            ++q;
            qbase[q] = (BT)(relative ? b - lo : b);
            for (int j = 0; j < 4; ++j) qval[4 * q + j] = real(0);
        }
        qval[4 * q + (c - b)] = (real)pval[k];
        last = c;
    }
}

// ------------------------------------------------- windows format (8, 4, 2, 1)
//
// Each row's off-diagonal entries (neuron-relative columns, increasing) are
// covered by windows of 8, 4, 2 or 1 consecutive columns: one 16-bit base per
// window and the window's values (zeros where a column is not kept), grouped by
// width within the row.  Walking the row, the window opened at the first
// uncovered entry c is the width with the fewest bytes per entry it covers (2 B
// base + width values; ties go to the wider window).  Windows may reach up to 7
// columns past the neuron's last segment, where the kernel keeps x at zero.
template <typename real>
__device__ __forceinline__ int window_width(const int32_t* pcol, int64_t k, int64_t end, int64_t row,
                                            int64_t* next) {
    const int widths[4] = {8, 4, 2, 1};
    const int64_t c = pcol[k];
    int best = -1;
    double best_per = 0.0;
    int64_t best_next = k + 1;
    for (int w = 0; w < 4; ++w) {
        int64_t j = k, cnt = 0;
        while (j < end && (pcol[j] == row || pcol[j] < c + widths[w])) {
            if (pcol[j] != row) ++cnt;
            ++j;
        }
        const double per = (2.0 + (double)widths[w] * sizeof(real)) / (double)cnt;
        if (best < 0 || per < best_per - 1e-12) { best = w; best_per = per; best_next = j; }
    }
    *next = best_next;
    return best;
}

// Per row: its window count of each width; flags[0] |= 1 when a row's columns
// do not increase (the format needs them sorted).
template <typename real>
__global__ void window_count_kernel(int64_t n, const int64_t* prow, const int32_t* pcol, int32_t* cnt,
                                    int* flags) {
    const int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (r >= n) return;
    int32_t c4[4] = {0, 0, 0, 0};
    const int64_t end = prow[r + 1];
    for (int64_t k = prow[r] + 1; k < end; ++k)
        if (pcol[k] <= pcol[k - 1]) { atomicOr(flags, 1); break; }
    int64_t k = prow[r];
    while (k < end && pcol[k] == r) ++k;
    while (k < end) {
        int64_t next;
        ++c4[window_width<real>(pcol, k, end, r, &next)];
        k = next;
        while (k < end && pcol[k] == r) ++k;
    }
    for (int w = 0; w < 4; ++w) cnt[4 * r + w] = c4[w];
}

// Writes row r's windows into its blocks: values of the 8-, 4-, 2- then 1-wide
// windows from 4 * d.x, bases in the same order from d.y.
template <typename real>
__global__ void window_fill_kernel(int64_t n, const int64_t* row_lo, const int64_t* prow, const int32_t* pcol,
                                   const double* pval, const uint4* desc, uint16_t* wbase, real* wval) {
    const int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (r >= n) return;
    const int widths[4] = {8, 4, 2, 1};
    const uint4 d = desc[r];
    const uint32_t cnt[4] = {d.z & 0xffffu, d.z >> 16, d.w & 0xffffu, d.w >> 16};
    int64_t voff[4], boff[4];
    voff[0] = 4 * (int64_t)d.x;
    boff[0] = d.y;
    for (int w = 1; w < 4; ++w) {
        voff[w] = voff[w - 1] + (int64_t)widths[w - 1] * cnt[w - 1];
        boff[w] = boff[w - 1] + cnt[w - 1];
    }
    const int64_t lo = row_lo[r], end = prow[r + 1];
    int64_t k = prow[r];
    while (k < end && pcol[k] == r) ++k;
    while (k < end) {
        int64_t next;
        const int w = window_width<real>(pcol, k, end, r, &next);
        const int64_t c = pcol[k];
        wbase[boff[w]++] = (uint16_t)(c - lo);
        real* v = wval + voff[w];
        voff[w] += widths[w];
        for (int j = 0; j < widths[w]; ++j) v[j] = real(0);
        for (int64_t e = k; e < next; ++e)
            if (pcol[e] != r) v[pcol[e] - c] = (real)pval[e];
        k = next;
        while (k < end && pcol[k] == r) ++k;
    }
}

static void free_windows(nw_ctx* ctx) {
    dev_free(ctx->win_row);
    dev_free(ctx->win_base);
    dev_free(ctx->win_val);
    for (int w = 0; w < 4; ++w) ctx->nwin[w] = 0;
    ctx->win_slots = 0;
    ctx->win_ok = false;
}

int ensure_windows(nw_ctx* ctx) {
    if (ctx->win_ok) return NW_OK;
    if (!ctx->b_ok) return fail(ctx, NW_ERR_LIMIT, "windows format: needs the batched format (neurons <= 65,535)");
    const int64_t n = ctx->n_seg;
    free_windows(ctx);
    DevBuf d_cnt, d_flag, d_lo;
    int rc = NW_OK;
    do {
        if ((rc = dev_alloc(ctx, d_cnt, 16 * n)) != NW_OK) break;
        if ((rc = dev_alloc(ctx, d_flag, 4)) != NW_OK) break;
        cudaError_t e = cudaMemsetAsync(d_flag.ptr, 0, 4, ctx->stream);
        if (e != cudaSuccess) { rc = cuda_fail(ctx, e, "windows format count"); break; }
        const unsigned blocks = (unsigned)((n + 127) / 128);
        if (ctx->precision == NW_F64)
            window_count_kernel<double><<<blocks, 128, 0, ctx->stream>>>(
                n, ctx->p_rowptr.as<int64_t>(), ctx->p_col.as<int32_t>(), d_cnt.as<int32_t>(), d_flag.as<int>());
        else
            window_count_kernel<float><<<blocks, 128, 0, ctx->stream>>>(
                n, ctx->p_rowptr.as<int64_t>(), ctx->p_col.as<int32_t>(), d_cnt.as<int32_t>(), d_flag.as<int>());
        std::vector<int32_t> cnt(4 * n);
        int flag = 0;
        cudaMemcpyAsync(cnt.data(), d_cnt.ptr, 16 * n, cudaMemcpyDeviceToHost, ctx->stream);
        cudaMemcpyAsync(&flag, d_flag.ptr, 4, cudaMemcpyDeviceToHost, ctx->stream);
        e = cudaStreamSynchronize(ctx->stream);
        if (e != cudaSuccess) { rc = cuda_fail(ctx, e, "windows format count"); break; }
        if (flag) { rc = fail(ctx, NW_ERR_STATE, "windows format: propagator rows are not sorted by column"); break; }
        // Row descriptors: value blocks rounded up to 4 values, bases back to back.
        std::vector<uint32_t> desc(4 * std::max<int64_t>(n, 1), 0);
        uint64_t vq = 0, nb = 0, tot[4] = {0, 0, 0, 0};
        for (int64_t i = 0; i < n && rc == NW_OK; ++i) {
            const int32_t* c = &cnt[4 * i];
            if (vq > UINT32_MAX || nb > UINT32_MAX) {
                rc = fail(ctx, NW_ERR_LIMIT, "windows format: more than 2^32 windows or value quads");
                break;
            }
            desc[4 * i] = (uint32_t)vq;
            desc[4 * i + 1] = (uint32_t)nb;
            desc[4 * i + 2] = (uint32_t)c[0] | ((uint32_t)c[1] << 16);
            desc[4 * i + 3] = (uint32_t)c[2] | ((uint32_t)c[3] << 16);
            vq += (uint64_t)(8 * c[0] + 4 * c[1] + 2 * c[2] + c[3] + 3) / 4;
            nb += (uint64_t)(c[0] + c[1] + c[2] + c[3]);
            for (int w = 0; w < 4; ++w) tot[w] += (uint64_t)c[w];
        }
        if (rc != NW_OK) break;
        for (int w = 0; w < 4; ++w) ctx->nwin[w] = (int64_t)tot[w];
        ctx->win_slots = (int64_t)(4 * vq);
        if ((rc = dev_alloc(ctx, ctx->win_row, 16 * std::max<int64_t>(n, 1))) != NW_OK) break;
        if ((rc = dev_alloc(ctx, ctx->win_base, 2 * std::max<uint64_t>(nb, 8))) != NW_OK) break;
        const size_t vbytes = (size_t)ctx->precision * 4 * std::max<uint64_t>(vq, 1);
        if ((rc = dev_alloc(ctx, ctx->win_val, vbytes)) != NW_OK) break;
        std::vector<int64_t> lo(n);
        for (int64_t j = 0; j < ctx->n_neuron; ++j)
            for (int64_t i = ctx->h_neuron_start[j]; i < ctx->h_neuron_start[j + 1]; ++i) lo[i] = ctx->h_neuron_start[j];
        if ((rc = dev_alloc(ctx, d_lo, 8 * std::max<int64_t>(n, 1))) != NW_OK) break;
        cudaMemsetAsync(ctx->win_val.ptr, 0, vbytes, ctx->stream);        // block padding reads as zero
        cudaMemcpyAsync(ctx->win_row.ptr, desc.data(), 16 * n, cudaMemcpyHostToDevice, ctx->stream);
        cudaMemcpyAsync(d_lo.ptr, lo.data(), 8 * n, cudaMemcpyHostToDevice, ctx->stream);
        if (ctx->precision == NW_F64)
            window_fill_kernel<double><<<blocks, 128, 0, ctx->stream>>>(
                n, d_lo.as<int64_t>(), ctx->p_rowptr.as<int64_t>(), ctx->p_col.as<int32_t>(), ctx->p_val.as<double>(),
                ctx->win_row.as<uint4>(), ctx->win_base.as<uint16_t>(), ctx->win_val.as<double>());
        else
            window_fill_kernel<float><<<blocks, 128, 0, ctx->stream>>>(
                n, d_lo.as<int64_t>(), ctx->p_rowptr.as<int64_t>(), ctx->p_col.as<int32_t>(), ctx->p_val.as<double>(),
                ctx->win_row.as<uint4>(), ctx->win_base.as<uint16_t>(), ctx->win_val.as<float>());
        e = cudaStreamSynchronize(ctx->stream);
        if (e != cudaSuccess) { rc = cuda_fail(ctx, e, "windows format fill"); break; }
        ctx->win_ok = true;
    } while (0);
    dev_free(d_cnt); dev_free(d_flag); dev_free(d_lo);
    if (rc != NW_OK) free_windows(ctx);
    return rc;
}

void free_quads(nw_ctx* ctx) {
    free_windows(ctx);
    dev_free(ctx->neuron_narrow);
    ctx->narrow_for = -1;
    for (DevBuf* b : {&ctx->q_rowptr, &ctx->q_base, &ctx->q_val, &ctx->wq_rowptr, &ctx->wq_base, &ctx->wq_val})
        dev_free(*b);
    ctx->q_ok = ctx->wq_ok = false;
    ctx->nq = ctx->nwq = 0;
}

// Quads of the FP64 CSR: neuron-relative 16-bit bases (batched path) or global
// 32-bit bases (wide path; windows of neurons of fewer than 4 segments may
// reach into the neighbouring segments, whose weights are zero).
template <typename BT>
static int build_quads(nw_ctx* ctx, bool relative, DevBuf& R, DevBuf& B, DevBuf& V, int64_t* nq_out,
                       std::vector<int64_t>* qrow_out = nullptr) {
    const int64_t n = ctx->n_seg;
    std::vector<int64_t> lo(n), hi(n);
    for (int64_t j = 0; j < ctx->n_neuron; ++j) {
        int64_t l = ctx->h_neuron_start[j], h = ctx->h_neuron_start[j + 1];
        if (!relative) {
            h = std::min<int64_t>(std::max<int64_t>(h, l + 4), n);
            l = std::min<int64_t>(l, h - 4);
        }
        for (int64_t i = ctx->h_neuron_start[j]; i < ctx->h_neuron_start[j + 1]; ++i) { lo[i] = l; hi[i] = h; }
    }
    DevBuf d_lo, d_hi, d_cnt;
    auto cleanup = [&]() { dev_free(d_lo); dev_free(d_hi); dev_free(d_cnt); };
    int rc = NW_OK;
    do {
        if ((rc = dev_alloc(ctx, d_lo, 8 * n)) != NW_OK) break;
        if ((rc = dev_alloc(ctx, d_hi, 8 * n)) != NW_OK) break;
        if ((rc = dev_alloc(ctx, d_cnt, 8 * n)) != NW_OK) break;
        cudaMemcpyAsync(d_lo.ptr, lo.data(), 8 * n, cudaMemcpyHostToDevice, ctx->stream);
        cudaMemcpyAsync(d_hi.ptr, hi.data(), 8 * n, cudaMemcpyHostToDevice, ctx->stream);
        quad_count_kernel<<<(unsigned)((n + 127) / 128), 128, 0, ctx->stream>>>(
            n, d_lo.as<int64_t>(), d_hi.as<int64_t>(), ctx->p_rowptr.as<int64_t>(), ctx->p_col.as<int32_t>(),
            d_cnt.as<int64_t>());
        std::vector<int64_t> cnt(n), qrow(n + 1, 0);
        cudaMemcpyAsync(cnt.data(), d_cnt.ptr, 8 * n, cudaMemcpyDeviceToHost, ctx->stream);
        cudaError_t e = cudaStreamSynchronize(ctx->stream);
        if (e != cudaSuccess) { rc = cuda_fail(ctx, e, "quad format count"); break; }
        for (int64_t i = 0; i < n; ++i) qrow[i + 1] = qrow[i] + cnt[i];
        const int64_t nq = qrow[n];
        if ((rc = dev_alloc(ctx, R, 8 * (n + 1))) != NW_OK) break;
        if ((rc = dev_alloc(ctx, B, sizeof(BT) * std::max<int64_t>(nq, 8))) != NW_OK) break;
        if ((rc = dev_alloc(ctx, V, (size_t)ctx->precision * 4 * std::max<int64_t>(nq, 1))) != NW_OK) break;
        cudaMemcpyAsync(R.ptr, qrow.data(), 8 * (n + 1), cudaMemcpyHostToDevice, ctx->stream);
        if (ctx->precision == NW_F64)
            quad_fill_kernel<double, BT><<<(unsigned)((n + 127) / 128), 128, 0, ctx->stream>>>(
                n, d_lo.as<int64_t>(), d_hi.as<int64_t>(), ctx->p_rowptr.as<int64_t>(), ctx->p_col.as<int32_t>(),
                ctx->p_val.as<double>(), R.as<int64_t>(), B.as<BT>(), V.as<double>(), relative ? 1 : 0);
        else
            quad_fill_kernel<float, BT><<<(unsigned)((n + 127) / 128), 128, 0, ctx->stream>>>(
                n, d_lo.as<int64_t>(), d_hi.as<int64_t>(), ctx->p_rowptr.as<int64_t>(), ctx->p_col.as<int32_t>(),
                ctx->p_val.as<double>(), R.as<int64_t>(), B.as<BT>(), V.as<float>(), relative ? 1 : 0);
        e = cudaStreamSynchronize(ctx->stream);
        if (e != cudaSuccess) { rc = cuda_fail(ctx, e, "quad format fill"); break; }
        *nq_out = nq;
        if (qrow_out) qrow_out->swap(qrow);
    } while (0);
    cleanup();
    return rc;
}

int ensure_quads(nw_ctx* ctx) {
    if (ctx->q_ok) return NW_OK;
    if (!ctx->b_ok) return fail(ctx, NW_ERR_LIMIT, "quad format: needs the batched format (neurons <= 65,535)");
    std::vector<int64_t> qrow;
    NW_CHECK(build_quads<uint16_t>(ctx, true, ctx->q_rowptr, ctx->q_base, ctx->q_val, &ctx->nq, &qrow));
    ctx->h_neuron_qpr.assign(ctx->n_neuron, 0.f);
    for (int64_t j = 0; j < ctx->n_neuron; ++j) {
        const int64_t a = ctx->h_neuron_start[j], b = ctx->h_neuron_start[j + 1];
        if (b > a) ctx->h_neuron_qpr[j] = (float)((double)(qrow[b] - qrow[a]) / (double)(b - a));
    }
    ctx->narrow_for = -1;
    ctx->q_ok = true;
    return NW_OK;
}

// Per-neuron flags of the quad format's narrow rows (mean quads per row below
// lanes_split), rebuilt when the threshold or the format changes.
int ensure_narrow(nw_ctx* ctx) {
    if (ctx->lanes_split <= 0 || !ctx->q_ok) return NW_OK;
    if (ctx->narrow_for == ctx->lanes_split && ctx->neuron_narrow.ptr) return NW_OK;
    std::vector<uint8_t> f(std::max<int64_t>(ctx->n_neuron, 1), 0);
    for (int64_t j = 0; j < ctx->n_neuron; ++j) f[j] = ctx->h_neuron_qpr[j] < (float)ctx->lanes_split ? 1 : 0;
    if (!ctx->neuron_narrow.ptr) NW_CHECK(dev_alloc(ctx, ctx->neuron_narrow, f.size()));
    NW_CUDA(ctx, cudaMemcpyAsync(ctx->neuron_narrow.ptr, f.data(), f.size(), cudaMemcpyHostToDevice, ctx->stream));
    NW_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    ctx->narrow_for = ctx->lanes_split;
    return NW_OK;
}

int ensure_wide_quads(nw_ctx* ctx) {
    if (ctx->wq_ok) return NW_OK;
    if (ctx->n_seg < 4) return fail(ctx, NW_ERR_LIMIT, "quad format: fewer than 4 segments");
    NW_CHECK(ensure_wide(ctx));                 // the leak comes with the wide row format
    NW_CHECK(build_quads<int32_t>(ctx, false, ctx->wq_rowptr, ctx->wq_base, ctx->wq_val, &ctx->nwq));
    ctx->wq_ok = true;
    return NW_OK;
}

// Called whenever the FP64 propagator changes: rebuilds the batched format (if
// every neuron fits its 16-bit columns) and drops the wide, pair and quad
// formats until next used.
int propagator_to_batched(nw_ctx* ctx) {
    free_wide(ctx);
    free_flux(ctx);
    free_quads(ctx);
    for (DevBuf* b : {&ctx->b_rowptr, &ctx->b_col, &ctx->b_val, &ctx->b_leak}) dev_free(*b);
    ctx->b_ok = false;
    ctx->nnz_b = 0;
    if (ctx->max_neuron > 65535) return NW_OK;
    NW_CHECK(csr_to_rows<uint16_t>(ctx, ctx->p_rowptr, ctx->p_col, ctx->p_val, true, ctx->b_rowptr, ctx->b_col,
                                   ctx->b_val, ctx->b_leak, &ctx->nnz_b));
    ctx->b_ok = true;
    return NW_OK;
}

int ensure_wide(nw_ctx* ctx) {
    if (ctx->w_ok) return NW_OK;
    NW_CHECK(csr_to_rows<int32_t>(ctx, ctx->p_rowptr, ctx->p_col, ctx->p_val, false, ctx->w_rowptr, ctx->w_col,
                                  ctx->w_val, ctx->w_leak, &ctx->nnz_w));
    ctx->w_ok = true;
    return NW_OK;
}

}  // namespace nw
