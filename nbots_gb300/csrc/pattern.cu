// Device build of the structures nbots derives from a mesh before assembly:
//   - the CSR pattern of nb_sparse_create(graph, NULL, 2) (sparse.c:20-60)
//     over the nodal graph of nb_mesh2D_load_graph(NB_NODES_LINKED_BY_ELEMS)
//     (load_graph.c:72-96, 230-328): each node links to both ends of its
//     edges and, in an element of more than three nodes, to the nen - 3
//     corners opposite it; its two rows list (2w, 2w+1) for every linked node
//     w and itself, ascending;
//   - the node -> (element, local node) incidence in ascending element order
//     that the row-gather assembly walks;
//   - the slice plan of the 2x2-block layout (bsr.cu).
// All of it is integer work: counts by atomic increments (order-free),
// offsets by exclusive scans, lists filled through atomic cursors and then
// sorted per node, so the result does not depend on the order in which the
// atomics land and equals the host build (nbg_host_pattern,
// nbg_host_incidence, nbg_bsr_plan) word for word.
#include <cstdint>

#include "common.cuh"

using namespace nbg;

namespace {

constexpr int kScanThreads = 1024;
constexpr int kScanItems = 2 * kScanThreads;  // per block

inline unsigned nblk(uint64_t n, unsigned t) { return (unsigned)((n + t - 1) / t); }

// Exclusive scan of one block's kScanItems values; writes local offsets and
// the block total.
__global__ void __launch_bounds__(kScanThreads)
    k_scan_block(const uint32_t* __restrict__ in, uint32_t* __restrict__ out, uint32_t n,
                 uint32_t* __restrict__ block_sum) {
    __shared__ uint32_t warp_tot[kScanThreads / 32];
    const uint32_t base = blockIdx.x * (uint32_t)kScanItems;
    const uint32_t i0 = base + 2 * threadIdx.x;
    const uint32_t a = i0 < n ? in[i0] : 0u, b = i0 + 1 < n ? in[i0 + 1] : 0u;
    const uint32_t t = a + b;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    uint32_t incl = t;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t y = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += y;
    }
    if (lane == 31) warp_tot[warp] = incl;
    __syncthreads();
    if (warp == 0) {
        uint32_t w = warp_tot[lane];
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t y = __shfl_up_sync(0xffffffffu, w, o);
            if (lane >= o) w += y;
        }
        warp_tot[lane] = w;  // inclusive over warps
    }
    __syncthreads();
    const uint32_t before = (warp ? warp_tot[warp - 1] : 0u) + incl - t;
    if (i0 < n) out[i0] = before;
    if (i0 + 1 < n) out[i0 + 1] = before + a;
    if (threadIdx.x == kScanThreads - 1) block_sum[blockIdx.x] = warp_tot[31];
}

__global__ void k_scan_add(uint32_t* __restrict__ out, uint32_t n,
                           const uint32_t* __restrict__ block_off) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) out[i] += block_off[i / kScanItems];
}

__global__ void k_set_total(uint32_t* __restrict__ out, uint32_t n,
                            const uint32_t* __restrict__ total) {
    out[n] = total[0];
}

// Every connectivity and edge index is a node of the mesh.
__global__ void k_check(uint32_t n_conn, const uint32_t* __restrict__ conn, uint32_t n_edg2,
                        const uint32_t* __restrict__ edg, uint32_t N_nod, int* bad) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n_conn && conn[i] >= N_nod) atomicExch(bad, 1);
    if (i < n_edg2 && edg[i] >= N_nod) atomicExch(bad, 1);
}

__global__ void k_count_edges(uint32_t N_edg, const uint32_t* __restrict__ edg,
                              uint32_t* __restrict__ deg) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= N_edg) return;
    atomicAdd(&deg[edg[2 * (size_t)i]], 1u);
    atomicAdd(&deg[edg[2 * (size_t)i + 1]], 1u);
}

__global__ void k_count_elems(uint32_t n_conn, uint32_t nen, const uint32_t* __restrict__ conn,
                              uint32_t* __restrict__ deg, uint32_t* __restrict__ inc_cnt) {
    const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n_conn) return;
    atomicAdd(&inc_cnt[conn[t]], 1u);
    if (nen > 3) atomicAdd(&deg[conn[t]], nen - 3);
}

// Per node: 2 (deg + 1) columns in each of its two rows.
__global__ void k_node_len(uint32_t N_nod, const uint32_t* __restrict__ deg,
                           uint32_t* __restrict__ len) {
    const uint32_t v = blockIdx.x * blockDim.x + threadIdx.x;
    if (v < N_nod) len[v] = 4u * (deg[v] + 1u);
}

__global__ void k_row_ptr(uint32_t N_nod, const uint32_t* __restrict__ deg,
                          const uint32_t* __restrict__ base, uint32_t* __restrict__ row_ptr) {
    const uint32_t v = blockIdx.x * blockDim.x + threadIdx.x;
    if (v > N_nod) return;
    if (v == N_nod) {
        row_ptr[2 * (size_t)N_nod] = base[N_nod];
        return;
    }
    row_ptr[2 * (size_t)v] = base[v];
    row_ptr[2 * (size_t)v + 1] = base[v] + 2u * (deg[v] + 1u);
}

// Linked nodes, unsorted, at nbr[base[v] / 4 + cursor].
__global__ void k_fill_edges(uint32_t N_edg, const uint32_t* __restrict__ edg,
                             const uint32_t* __restrict__ base, uint32_t* __restrict__ cur,
                             uint32_t* __restrict__ nbr) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= N_edg) return;
    const uint32_t a = edg[2 * (size_t)i], b = edg[2 * (size_t)i + 1];
    nbr[base[a] / 4 + atomicAdd(&cur[a], 1u)] = b;
    nbr[base[b] / 4 + atomicAdd(&cur[b], 1u)] = a;
}

__global__ void k_fill_elems(uint32_t N_elem, uint32_t nen, const uint32_t* __restrict__ conn,
                             const uint32_t* __restrict__ base, uint32_t* __restrict__ cur,
                             uint32_t* __restrict__ nbr, const uint32_t* __restrict__ inc_ptr,
                             uint32_t* __restrict__ inc_cur, uint32_t* __restrict__ inc_elem,
                             uint8_t* __restrict__ inc_local) {
    const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= N_elem * nen) return;
    const uint32_t e = t / nen, i = t % nen;
    const uint32_t v = conn[t];
    const uint32_t p = inc_ptr[v] + atomicAdd(&inc_cur[v], 1u);
    inc_elem[p] = e;
    inc_local[p] = (uint8_t)i;
    for (uint32_t j = 0; j + 3 < nen; j++)
        nbr[base[v] / 4 + atomicAdd(&cur[v], 1u)] = conn[(size_t)e * nen + (i + j + 2) % nen];
}

// Per node: append itself, sort its links, write its two rows.
__global__ void k_rows(uint32_t N_nod, const uint32_t* __restrict__ deg,
                       const uint32_t* __restrict__ base, uint32_t* __restrict__ nbr,
                       uint32_t* __restrict__ col_idx) {
    const uint32_t v = blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= N_nod) return;
    const uint32_t d = deg[v] + 1u;
    uint32_t* l = nbr + base[v] / 4;
    l[d - 1] = v;
    for (uint32_t a = 1; a < d; a++) {  // insertion sort: a few to a few dozen links
        const uint32_t x = l[a];
        uint32_t b = a;
        while (b > 0 && l[b - 1] > x) {
            l[b] = l[b - 1];
            b--;
        }
        l[b] = x;
    }
    uint32_t* r0 = col_idx + base[v];
    uint32_t* r1 = r0 + 2 * d;
    for (uint32_t a = 0; a < d; a++) {
        r0[2 * a] = r1[2 * a] = 2u * l[a];
        r0[2 * a + 1] = r1[2 * a + 1] = 2u * l[a] + 1u;
    }
}

// Per node: its incidence in ascending (element, local node) order.
__global__ void k_sort_inc(uint32_t N_nod, const uint32_t* __restrict__ inc_ptr,
                           uint32_t* __restrict__ inc_elem, uint8_t* __restrict__ inc_local) {
    const uint32_t v = blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= N_nod) return;
    const uint32_t b0 = inc_ptr[v], n = inc_ptr[v + 1] - b0;
    uint32_t* e = inc_elem + b0;
    uint8_t* l = inc_local + b0;
    for (uint32_t a = 1; a < n; a++) {
        const uint32_t xe = e[a];
        const uint8_t xl = l[a];
        uint32_t b = a;
        while (b > 0 && (e[b - 1] > xe || (e[b - 1] == xe && l[b - 1] > xl))) {
            e[b] = e[b - 1];
            l[b] = l[b - 1];
            b--;
        }
        e[b] = xe;
        l[b] = xl;
    }
}

// Width of each 32-node slice of the block layout: its longest node row,
// in 2x2 blocks.
__global__ void k_slice_width(uint32_t N_nod, uint32_t S, const uint32_t* __restrict__ deg,
                              uint32_t* __restrict__ w) {
    const uint32_t s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= S) return;
    uint32_t m = 0;
    for (uint32_t v = 32 * s; v < N_nod && v < 32 * s + 32; v++) m = max(m, deg[v] + 1u);
    w[s] = m;
}

// SELL-C-sigma order: one block per window of sigma nodes; each node's place
// is the number of nodes of its window with a longer row, or as long a row
// and a smaller index.
__global__ void __launch_bounds__(1024)
    k_sigma_perm(uint32_t N_nod, uint32_t sigma, const uint32_t* __restrict__ rp,
                 uint32_t* __restrict__ perm, uint32_t* __restrict__ iperm) {
    __shared__ uint32_t w[1024];
    const uint32_t s0 = blockIdx.x * sigma, t = threadIdx.x;
    const uint32_t n = min(sigma, N_nod - s0);
    const uint32_t v = s0 + t;
    const uint32_t wv = t < n ? rp[2 * (size_t)v + 1] - rp[2 * (size_t)v] : 0u;
    w[t] = wv;
    __syncthreads();
    if (t >= n) return;
    uint32_t rank = 0;
    for (uint32_t u = 0; u < n; u++) rank += (w[u] > wv) || (w[u] == wv && u < t);
    perm[s0 + rank] = v;
    iperm[v] = s0 + rank;
}

__global__ void k_slice_width_perm(uint32_t N_nod, uint32_t S, const uint32_t* __restrict__ perm,
                                   const uint32_t* __restrict__ rp, uint32_t* __restrict__ w) {
    const uint32_t s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= S) return;
    uint32_t m = 0;
    for (uint32_t i = 32 * s; i < N_nod && i < 32 * s + 32; i++) {
        const uint32_t v = perm[i];
        m = max(m, (rp[2 * (size_t)v + 1] - rp[2 * (size_t)v]) / 2);
    }
    w[s] = m;
}

// Exclusive scan of n values into out[0..n], out[n] the total; tmp needs
// scan_tmp_words(n) words.
size_t scan_tmp_words(uint32_t n) {
    size_t words = 0;
    while (n > (uint32_t)kScanItems) {
        const uint32_t nb = nblk(n, kScanItems);
        words += 2 * (size_t)nb + 1;
        n = nb;
    }
    return words + 1;
}

int scan_exclusive(const uint32_t* in, uint32_t* out, uint32_t n, uint32_t* tmp,
                   cudaStream_t s) {
    const uint32_t nb = n ? nblk(n, kScanItems) : 1;
    uint32_t* sums = tmp;
    k_scan_block<<<nb, kScanThreads, 0, s>>>(in, out, n, sums);
    NBG_CHECK(cudaGetLastError());
    if (nb == 1) {
        k_set_total<<<1, 1, 0, s>>>(out, n, sums);
        NBG_CHECK(cudaGetLastError());
        return NBG_OK;
    }
    uint32_t* offs = tmp + nb;  // nb + 1 words
    int rc = scan_exclusive(sums, offs, nb, tmp + 2 * (size_t)nb + 1, s);
    if (rc != NBG_OK) return rc;
    k_scan_add<<<nblk(n, 256), 256, 0, s>>>(out, n, offs);
    NBG_CHECK(cudaGetLastError());
    k_set_total<<<1, 1, 0, s>>>(out, n, offs + nb);
    NBG_CHECK(cudaGetLastError());
    return NBG_OK;
}

}  // namespace

extern "C" int nbg_pattern_dev(uint32_t nen, uint32_t N_nod, uint32_t N_elem, uint32_t N_edg,
                               const uint32_t* conn, const uint32_t* edg, uint32_t* row_ptr,
                               uint32_t** col_idx, uint64_t* nnz, uint32_t* inc_ptr,
                               uint32_t* inc_elem, uint8_t* inc_local, uint32_t* slice_off,
                               void* stream) {
    if ((nen != 3 && nen != 4) || N_nod == 0 || !col_idx || !nnz) return NBG_ERR_ARG;
    if ((uint64_t)N_elem * nen > 0xffffffffull || 2ull * N_edg > 0xffffffffull)
        return NBG_ERR_ARG;
    *col_idx = nullptr;
    *nnz = 0;
    cudaStream_t s = (cudaStream_t)stream;
    const uint32_t n_conn = N_elem * nen, S = (N_nod + 31) / 32;
    const uint32_t big = N_nod > S ? N_nod : S;
    // scratch: deg, inc count, len, base, cursor, inc cursor (N_nod + 1 each),
    // scan temporaries, the node link lists, and a flag
    const size_t tmp_words = scan_tmp_words(big + 1);
    uint32_t* ws = nullptr;
    const size_t ws_words = 6 * ((size_t)N_nod + 1) + tmp_words + 1;
    NBG_CHECK(cudaMalloc(&ws, 4 * ws_words));
    uint32_t *deg = ws, *icnt = deg + N_nod + 1, *len = icnt + N_nod + 1;
    uint32_t *base = len + N_nod + 1, *cur = base + N_nod + 1, *icur = cur + N_nod + 1;
    uint32_t* tmp = icur + N_nod + 1;
    int* bad = (int*)(tmp + tmp_words);
    uint32_t* nbr = nullptr;
    uint32_t* ci = nullptr;
    int rc = NBG_OK;
    int bad_h = 0;
    uint32_t total = 0;
    cudaError_t e = cudaMemsetAsync(ws, 0, 4 * ws_words, s);
    const unsigned T = 256;
    const uint32_t n_chk = n_conn > 2 * N_edg ? n_conn : 2 * N_edg;
    if (e == cudaSuccess && n_chk) {
        k_check<<<nblk(n_chk, T), T, 0, s>>>(n_conn, conn, 2 * N_edg, edg, N_nod, bad);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaMemcpyAsync(&bad_h, bad, 4, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) {
        rc = nbg_cuda_error(e);
        goto done;
    }
    if (bad_h) {
        rc = nbg_error_text(NBG_ERR_ARG, "nbg_pattern_dev: a node index is out of range");
        goto done;
    }
    if (N_edg) k_count_edges<<<nblk(N_edg, T), T, 0, s>>>(N_edg, edg, deg);
    if (n_conn) k_count_elems<<<nblk(n_conn, T), T, 0, s>>>(n_conn, nen, conn, deg, icnt);
    k_node_len<<<nblk(N_nod, T), T, 0, s>>>(N_nod, deg, len);
    if ((e = cudaGetLastError()) != cudaSuccess) {
        rc = nbg_cuda_error(e);
        goto done;
    }
    if ((rc = scan_exclusive(len, base, N_nod, tmp, s)) != NBG_OK) goto done;
    if ((rc = scan_exclusive(icnt, inc_ptr, N_nod, tmp, s)) != NBG_OK) goto done;
    k_row_ptr<<<nblk((uint64_t)N_nod + 1, T), T, 0, s>>>(N_nod, deg, base, row_ptr);
    e = cudaGetLastError();
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(&total, base + N_nod, 4, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) {
        rc = nbg_cuda_error(e);
        goto done;
    }
    e = cudaMalloc(&nbr, 4 * ((size_t)total / 4 + 1));
    if (e == cudaSuccess) e = cudaMalloc(&ci, 4 * ((size_t)total + 1));
    if (e != cudaSuccess) {
        rc = nbg_cuda_error(e);
        goto done;
    }
    if (N_edg) k_fill_edges<<<nblk(N_edg, T), T, 0, s>>>(N_edg, edg, base, cur, nbr);
    if (n_conn)
        k_fill_elems<<<nblk(n_conn, T), T, 0, s>>>(N_elem, nen, conn, base, cur, nbr, inc_ptr,
                                                   icur, inc_elem, inc_local);
    k_rows<<<nblk(N_nod, T), T, 0, s>>>(N_nod, deg, base, nbr, ci);
    k_sort_inc<<<nblk(N_nod, T), T, 0, s>>>(N_nod, inc_ptr, inc_elem, inc_local);
    if (slice_off) {
        k_slice_width<<<nblk(S, T), T, 0, s>>>(N_nod, S, deg, len);
        e = cudaGetLastError();
        if (e == cudaSuccess && (rc = scan_exclusive(len, slice_off, S, tmp, s)) != NBG_OK)
            goto done;
    }
    e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) {
        rc = nbg_cuda_error(e);
        goto done;
    }
    *col_idx = ci;
    ci = nullptr;
    *nnz = total;
done:
    if (ci) cudaFree(ci);
    if (nbr) cudaFree(nbr);
    cudaFree(ws);
    return rc;
}

extern "C" int nbg_bsr_plan_sigma_dev(uint32_t N_nod, const uint32_t* row_ptr, uint32_t sigma,
                                      uint32_t* perm, uint32_t* iperm, uint32_t* slice_off,
                                      void* stream) {
    if (N_nod == 0 || sigma == 0 || sigma > 1024 || !perm || !iperm || !slice_off)
        return NBG_ERR_ARG;
    cudaStream_t s = (cudaStream_t)stream;
    const uint32_t S = (N_nod + 31) / 32;
    const size_t tmp_words = scan_tmp_words(S);
    uint32_t* ws = nullptr;
    NBG_CHECK(cudaMalloc(&ws, 4 * ((size_t)S + tmp_words)));
    int rc = NBG_OK;
    k_sigma_perm<<<nblk(N_nod, sigma), sigma, 0, s>>>(N_nod, sigma, row_ptr, perm, iperm);
    k_slice_width_perm<<<nblk(S, 256), 256, 0, s>>>(N_nod, S, perm, row_ptr, ws);
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess) rc = scan_exclusive(ws, slice_off, S, ws + S, s);
    if (e == cudaSuccess && rc == NBG_OK) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) rc = nbg_cuda_error(e);
    cudaFree(ws);
    return rc;
}
