// Sparsity pattern and scatter-map construction (once per topology).
//
// Reproduces CompCol::buildInternalStructure (src/core/compcol.C:174-272): the
// pattern is the union of all location-array pairs, columns sorted per row.
// Two builders:
//   * mesh builder (element backend): node incidence -> node adjacency ("node
//     blocks") -> DOF rows. Free DOFs are numbered node-major, so sorted
//     neighbour nodes give sorted columns; each node block also gets the list of
//     (element, a, b) contributions in element order, which is the gather map
//     of the deterministic assembly.
//   * location-array builder (drop-in SparseMtrx path): the same on equations.
// No sort library and no floating-point atomics: counts use integer atomics,
// lists are put in a canonical order by a per-segment insertion sort.
#include <vector>

#include "internal.cuh"

namespace ogb {

namespace {

constexpr int MAX_NB = 128;     // node neighbours per node
constexpr int MAX_ROW = 512;    // columns per equation row (location-array builder)

__global__ void k_count_inc(int nelem, int nnpe, const int *__restrict__ conn, unsigned long long *cnt)
{
    int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (int64_t)nelem * nnpe) return;
    atomicAdd(cnt + conn[t], 1ull);
}

__global__ void k_fill_inc(int nelem, int nnpe, const int *__restrict__ conn, const int64_t *__restrict__ ptr,
                           unsigned int *fill, uint32_t *inc)
{
    int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (int64_t)nelem * nnpe) return;
    int e = (int)(t / nnpe), a = (int)(t % nnpe);
    int n = conn[t];
    unsigned int s = atomicAdd(fill + n, 1u);
    inc[ptr[n] + s] = ((uint32_t)e << 3) | (uint32_t)a;
}

template <class T>
__global__ void k_sort_segments(int64_t nseg, const int64_t *__restrict__ ptr, T *v)
{
    int64_t s = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= nseg) return;
    int64_t b = ptr[s], e = ptr[s + 1];
    for (int64_t i = b + 1; i < e; ++i) {
        T x = v[i];
        int64_t j = i - 1;
        while (j >= b && v[j] > x) {
            v[j + 1] = v[j];
            --j;
        }
        v[j + 1] = x;
    }
}

__device__ __forceinline__ int nfree_of(const int *eq, int ndofpn, int n)
{
    int c = 0;
    for (int d = 0; d < ndofpn; ++d) c += eq[(size_t)n * ndofpn + d] > 0;
    return c;
}

// Sorted unique neighbour nodes of node A (union over incident elements).
__device__ int gather_neighbours(int A, int nnpe, const int *__restrict__ conn, const int64_t *__restrict__ inc_ptr,
                                 const uint32_t *__restrict__ inc, int *nb, int *status)
{
    int cnt = 0;
    for (int64_t k = inc_ptr[A]; k < inc_ptr[A + 1]; ++k) {
        int e = (int)(inc[k] >> 3);
        for (int b = 0; b < nnpe; ++b) {
            int B = conn[(size_t)e * nnpe + b];
            // insert into sorted nb[0..cnt)
            int lo = 0, hi = cnt;
            while (lo < hi) {
                int mid = (lo + hi) >> 1;
                if (nb[mid] < B) lo = mid + 1; else hi = mid;
            }
            if (lo < cnt && nb[lo] == B) continue;
            if (cnt >= MAX_NB) {
                atomicCAS(status, DS_OK, DS_LIMIT);
                return cnt;
            }
            for (int j = cnt; j > lo; --j) nb[j] = nb[j - 1];
            nb[lo] = B;
            ++cnt;
        }
    }
    return cnt;
}

__global__ void k_count_nb(int nnodes, int nnpe, const int *conn, const int64_t *inc_ptr, const uint32_t *inc,
                           int64_t *nbcnt, int *status)
{
    int A = blockIdx.x * blockDim.x + threadIdx.x;
    if (A >= nnodes) return;
    int nb[MAX_NB];
    nbcnt[A] = gather_neighbours(A, nnpe, conn, inc_ptr, inc, nb, status);
}

// Per node A: neighbour list, column offsets of each block inside A's rows,
// contribution counts per block, row length and rows x length of the node.
__global__ void k_fill_nb(int nnodes, int nnpe, int ndofpn, const int *conn, const int *eq, const int64_t *inc_ptr,
                          const uint32_t *inc, const int64_t *nb_ptr, int *nb_col, int *nb_coloff, int *blk_node,
                          int64_t *cbcnt, int *node_rowlen, int64_t *node_nnz, int *status)
{
    int A = blockIdx.x * blockDim.x + threadIdx.x;
    if (A >= nnodes) return;
    int nb[MAX_NB];
    int cnt = gather_neighbours(A, nnpe, conn, inc_ptr, inc, nb, status);
    int64_t base = nb_ptr[A];
    int off = 0;
    for (int k = 0; k < cnt; ++k) {
        nb_col[base + k] = nb[k];
        nb_coloff[base + k] = off;
        blk_node[base + k] = A;
        cbcnt[base + k] = 0;
        off += nfree_of(eq, ndofpn, nb[k]);
    }
    node_rowlen[A] = off;
    node_nnz[A] = (int64_t)off * nfree_of(eq, ndofpn, A);
    for (int64_t k = inc_ptr[A]; k < inc_ptr[A + 1]; ++k) {
        int e = (int)(inc[k] >> 3);
        for (int b = 0; b < nnpe; ++b) {
            int B = conn[(size_t)e * nnpe + b];
            int lo = 0, hi = cnt;
            while (lo < hi) {
                int mid = (lo + hi) >> 1;
                if (nb[mid] < B) lo = mid + 1; else hi = mid;
            }
            cbcnt[base + lo] += 1;
        }
    }
}

__global__ void k_fill_contrib(int nnodes, int nnpe, const int *conn, const int64_t *inc_ptr, const uint32_t *inc,
                               const int64_t *nb_ptr, const int *nb_col, const int64_t *cb_ptr, uint32_t *cb)
{
    int A = blockIdx.x * blockDim.x + threadIdx.x;
    if (A >= nnodes) return;
    int64_t base = nb_ptr[A];
    int cnt = (int)(nb_ptr[A + 1] - base);
    int fill[MAX_NB];
    for (int k = 0; k < cnt; ++k) fill[k] = 0;
    for (int64_t k = inc_ptr[A]; k < inc_ptr[A + 1]; ++k) {   // elements ascending
        int e = (int)(inc[k] >> 3), a = (int)(inc[k] & 7u);
        for (int b = 0; b < nnpe; ++b) {
            int B = conn[(size_t)e * nnpe + b];
            int lo = 0, hi = cnt;
            while (lo < hi) {
                int mid = (lo + hi) >> 1;
                if (nb_col[base + mid] < B) lo = mid + 1; else hi = mid;
            }
            cb[cb_ptr[base + lo] + fill[lo]++] = ((uint32_t)e << 6) | ((uint32_t)a << 3) | (uint32_t)b;
        }
    }
}

// Row pointers, column indices and diagonal positions of the DOF-level CSR.
__global__ void k_fill_rows(int nnodes, int ndofpn, const int *eq, const int64_t *nb_ptr, const int *nb_col,
                            const int *nb_coloff, const int *node_rowlen, const int64_t *node_rowbase,
                            int64_t *rowptr, int *colind, int64_t *diagpos)
{
    int A = blockIdx.x * blockDim.x + threadIdx.x;
    if (A >= nnodes) return;
    int len = node_rowlen[A];
    int64_t base = node_rowbase[A];
    int ip = 0;
    for (int i = 0; i < ndofpn; ++i) {
        int r = eq[(size_t)A * ndofpn + i];
        if (r <= 0) continue;
        int64_t rb = base + (int64_t)ip * len;
        rowptr[r - 1] = rb;
        for (int64_t k = nb_ptr[A]; k < nb_ptr[A + 1]; ++k) {
            int B = nb_col[k];
            int jp = 0;
            for (int j = 0; j < ndofpn; ++j) {
                int c = eq[(size_t)B * ndofpn + j];
                if (c <= 0) continue;
                colind[rb + nb_coloff[k] + jp] = c - 1;
                if (B == A && j == i) diagpos[r - 1] = rb + nb_coloff[k] + jp;
                ++jp;
            }
        }
        ++ip;
    }
}

// Identity rows neq..npad-1 after the real entries (diagonal 1).
__global__ void k_pad_rows(int neq, int npad, int64_t nnz, int64_t *rowptr, int *colind, double *val, int64_t *diagpos)
{
    int r = neq + blockIdx.x * blockDim.x + threadIdx.x;
    if (r > npad) return;
    int64_t p = nnz + (r - neq);
    rowptr[r] = p;
    if (r < npad) {
        colind[p] = r;
        val[p] = 1.0;
        diagpos[r] = p;
    }
}

// ---- location-array builder (drop-in path) ---------------------------------
__global__ void k_loc_count_inc(int nelem, const int64_t *lptr, const int *loc, unsigned long long *cnt)
{
    int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= nelem) return;
    for (int64_t k = lptr[s]; k < lptr[s + 1]; ++k)
        if (loc[k] > 0) atomicAdd(cnt + (loc[k] - 1), 1ull);
}

__global__ void k_loc_fill_inc(int nelem, const int64_t *lptr, const int *loc, const int64_t *ptr, unsigned int *fill,
                               uint32_t *inc)
{
    int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= nelem) return;
    for (int64_t k = lptr[s]; k < lptr[s + 1]; ++k)
        if (loc[k] > 0) {
            int r = loc[k] - 1;
            unsigned int f = atomicAdd(fill + r, 1u);
            inc[ptr[r] + f] = (uint32_t)s;
        }
}

__device__ int gather_row(int r, const int64_t *lptr, const int *loc, const int64_t *inc_ptr, const uint32_t *inc,
                          int *cols, int *status)
{
    int cnt = 0;
    for (int64_t k = inc_ptr[r]; k < inc_ptr[r + 1]; ++k) {
        int s = (int)inc[k];
        for (int64_t q = lptr[s]; q < lptr[s + 1]; ++q) {
            int c = loc[q] - 1;
            if (c < 0) continue;
            int lo = 0, hi = cnt;
            while (lo < hi) {
                int mid = (lo + hi) >> 1;
                if (cols[mid] < c) lo = mid + 1; else hi = mid;
            }
            if (lo < cnt && cols[lo] == c) continue;
            if (cnt >= MAX_ROW) {
                atomicCAS(status, DS_OK, DS_LIMIT);
                return cnt;
            }
            for (int j = cnt; j > lo; --j) cols[j] = cols[j - 1];
            cols[lo] = c;
            ++cnt;
        }
    }
    return cnt;
}

__global__ void k_loc_count_row(int neq, const int64_t *lptr, const int *loc, const int64_t *inc_ptr,
                                const uint32_t *inc, int64_t *rowcnt, int *status)
{
    int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= neq) return;
    int cols[MAX_ROW];
    rowcnt[r] = gather_row(r, lptr, loc, inc_ptr, inc, cols, status);
}

__global__ void k_loc_fill_row(int neq, const int64_t *lptr, const int *loc, const int64_t *inc_ptr,
                               const uint32_t *inc, const int64_t *rowptr, int *colind, int64_t *diagpos, int *status)
{
    int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= neq) return;
    int cols[MAX_ROW];
    int cnt = gather_row(r, lptr, loc, inc_ptr, inc, cols, status);
    int64_t b = rowptr[r];
    diagpos[r] = -1;
    for (int k = 0; k < cnt; ++k) {
        colind[b + k] = cols[k];
        if (cols[k] == r) diagpos[r] = b + k;
    }
}

// ---- staged (host element matrix) assembly -----------------------------------
__device__ __forceinline__ int64_t find_pos(const int64_t *rowptr, const int *colind, int r, int c)
{
    int64_t lo = rowptr[r], hi = rowptr[r + 1] - 1;
    while (lo <= hi) {
        int64_t mid = (lo + hi) >> 1;
        int v = colind[mid];
        if (v < c) lo = mid + 1;
        else if (v > c) hi = mid - 1;
        else return mid;
    }
    return -1;
}

// One thread per (staged matrix s, column j): CompCol::assemble loops columns
// outer, rows inner (compcol.C:288-310).
__global__ void k_stage_count(int nst, const int64_t *lptr, const int *loc, const int64_t *rowptr, const int *colind,
                              unsigned int *cnt, int *status)
{
    int s = blockIdx.x;
    int64_t b = lptr[s];
    int n = (int)(lptr[s + 1] - b);
    for (int j = threadIdx.x; j < n; j += blockDim.x) {
        int cj = loc[b + j];
        if (cj <= 0) continue;
        for (int i = 0; i < n; ++i) {
            int ri = loc[b + i];
            if (ri <= 0) continue;
            int64_t p = find_pos(rowptr, colind, ri - 1, cj - 1);
            if (p < 0) { atomicCAS(status, DS_OK, DS_PATTERN); continue; }
            atomicAdd(cnt + p, 1u);
        }
    }
}

__global__ void k_stage_fill(int nst, const int64_t *lptr, const int *loc, const int64_t *keoff, const int64_t *rowptr,
                             const int *colind, const int64_t *cptr, unsigned int *fill, int64_t *src)
{
    int s = blockIdx.x;
    int64_t b = lptr[s];
    int n = (int)(lptr[s + 1] - b);
    for (int j = threadIdx.x; j < n; j += blockDim.x) {
        int cj = loc[b + j];
        if (cj <= 0) continue;
        for (int i = 0; i < n; ++i) {
            int ri = loc[b + i];
            if (ri <= 0) continue;
            int64_t p = find_pos(rowptr, colind, ri - 1, cj - 1);
            if (p < 0) continue;
            unsigned int f = atomicAdd(fill + p, 1u);
            src[cptr[p] + f] = keoff[s] + (int64_t)j * n + i;   // column-major index == reference order
        }
    }
}

__global__ void k_stage_apply(int64_t nnz, const int64_t *cptr, const int64_t *src, const double *ke, double *val)
{
    int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= nnz) return;
    int64_t b = cptr[p], e = cptr[p + 1];
    if (b == e) return;
    double acc = val[p];
    for (int64_t k = b; k < e; ++k) acc += ke[src[k]];
    val[p] = acc;
}

template <class T>
__global__ void k_u64_to_i64(int64_t n, const T *in, int64_t *out)
{
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) out[i] = (int64_t)in[i];
}

inline unsigned nblk(int64_t n) { return (unsigned)ceil_div(n > 0 ? n : 1, NTHREADS); }

}  // namespace

int build_incidence(ogb_ctx *ctx, int nnodes, int nelem, int nnpe, const int *conn, DBuf<int64_t> &inc_ptr,
                    DBuf<uint32_t> &inc)
{
    cudaStream_t st = ctx->stream;
    int64_t ntot = (int64_t)nelem * nnpe;
    DBuf<unsigned long long> cnt;
    OGB_CHECK(cnt.alloc(nnodes + 1));
    OGB_CUDA(cudaMemsetAsync(cnt.p, 0, (nnodes + 1) * sizeof(unsigned long long), st));
    k_count_inc<<<nblk(ntot), NTHREADS, 0, st>>>(nelem, nnpe, conn, cnt.p);
    OGB_CHECK(inc_ptr.alloc(nnodes + 1));
    k_u64_to_i64<<<nblk(nnodes + 1), NTHREADS, 0, st>>>(nnodes + 1, cnt.p, inc_ptr.p);
    count_launch(ctx, 2);
    int64_t total = 0;
    OGB_CHECK(exclusive_scan_i64(ctx, inc_ptr.p, inc_ptr.p, nnodes + 1, &total));
    OGB_CHECK(inc.alloc(total));
    DBuf<unsigned int> fill;
    OGB_CHECK(fill.alloc(nnodes));
    OGB_CUDA(cudaMemsetAsync(fill.p, 0, nnodes * sizeof(unsigned int), st));
    k_fill_inc<<<nblk(ntot), NTHREADS, 0, st>>>(nelem, nnpe, conn, inc_ptr.p, fill.p, inc.p);
    k_sort_segments<uint32_t><<<nblk(nnodes), NTHREADS, 0, st>>>(nnodes, inc_ptr.p, inc.p);
    count_launch(ctx, 2);
    OGB_CUDA(cudaGetLastError());
    OGB_CUDA(cudaStreamSynchronize(st));
    return OGB_OK;
}

int pad_matrix_rows(ogb_mtrx *m)
{
    int np = m->npad - m->neq;
    k_pad_rows<<<nblk(np + 1), NTHREADS, 0, m->ctx->stream>>>(m->neq, m->npad, m->nnz, m->rowptr.p, m->colind.p,
                                                               m->val.p, m->diagpos.p);
    count_launch(m->ctx);
    OGB_CUDA(cudaGetLastError());
    return OGB_OK;
}

static int alloc_matrix(ogb_mtrx *m, int neq, int64_t nnz)
{
    m->neq = neq;
    m->nnz = nnz;
    m->npad = (int)(ceil_div(neq > 0 ? neq : 1, CHUNK) * CHUNK);
    int64_t ntot = nnz + (m->npad - neq);
    OGB_CHECK(m->rowptr.alloc(m->npad + 1));
    OGB_CHECK(m->colind.alloc(ntot));
    OGB_CHECK(m->val.alloc(ntot));
    OGB_CHECK(m->diagpos.alloc(m->npad));
    OGB_CUDA(cudaMemsetAsync(m->val.p, 0, nnz * sizeof(double), m->ctx->stream));
    return OGB_OK;
}

int build_model_pattern(ogb_model *md, ogb_mtrx *m)
{
    ogb_ctx *ctx = md->ctx;
    cudaStream_t st = ctx->stream;
    int nn = md->nnodes;
    OGB_CUDA(cudaMemsetAsync(ctx->status.p, 0, sizeof(int), st));
    OGB_CHECK(build_incidence(ctx, nn, md->nelem, md->nnpe, md->conn.p, md->inc_ptr, md->inc));
    // node adjacency
    OGB_CHECK(md->nb_ptr.alloc(nn + 1));
    OGB_CUDA(cudaMemsetAsync(md->nb_ptr.p + nn, 0, sizeof(int64_t), st));
    k_count_nb<<<nblk(nn), NTHREADS, 0, st>>>(nn, md->nnpe, md->conn.p, md->inc_ptr.p, md->inc.p, md->nb_ptr.p,
                                              ctx->status.p);
    count_launch(ctx);
    int64_t nblocks = 0;
    OGB_CHECK(exclusive_scan_i64(ctx, md->nb_ptr.p, md->nb_ptr.p, nn + 1, &nblocks));
    OGB_CHECK(check_device_status(ctx, "node adjacency"));
    md->nblocks = nblocks;
    OGB_CHECK(md->nb_col.alloc(nblocks));
    OGB_CHECK(md->nb_coloff.alloc(nblocks));
    OGB_CHECK(md->blk_node.alloc(nblocks));
    OGB_CHECK(md->cb_ptr.alloc(nblocks + 1));
    OGB_CHECK(md->node_rowlen.alloc(nn));
    OGB_CHECK(md->node_rowbase.alloc(nn + 1));
    OGB_CUDA(cudaMemsetAsync(md->cb_ptr.p + nblocks, 0, sizeof(int64_t), st));
    OGB_CUDA(cudaMemsetAsync(md->node_rowbase.p + nn, 0, sizeof(int64_t), st));
    k_fill_nb<<<nblk(nn), NTHREADS, 0, st>>>(nn, md->nnpe, md->ndofpn, md->conn.p, md->eq.p, md->inc_ptr.p,
                                             md->inc.p, md->nb_ptr.p, md->nb_col.p, md->nb_coloff.p, md->blk_node.p,
                                             md->cb_ptr.p, md->node_rowlen.p, md->node_rowbase.p, ctx->status.p);
    count_launch(ctx);
    int64_t ncontrib = 0, nnz = 0;
    OGB_CHECK(exclusive_scan_i64(ctx, md->cb_ptr.p, md->cb_ptr.p, nblocks + 1, &ncontrib));
    OGB_CHECK(exclusive_scan_i64(ctx, md->node_rowbase.p, md->node_rowbase.p, nn + 1, &nnz));
    OGB_CHECK(md->cb.alloc(ncontrib));
    k_fill_contrib<<<nblk(nn), NTHREADS, 0, st>>>(nn, md->nnpe, md->conn.p, md->inc_ptr.p, md->inc.p, md->nb_ptr.p,
                                                  md->nb_col.p, md->cb_ptr.p, md->cb.p);
    count_launch(ctx);
    // DOF-level CSR
    OGB_CHECK(alloc_matrix(m, md->neq, nnz));
    k_fill_rows<<<nblk(nn), NTHREADS, 0, st>>>(nn, md->ndofpn, md->eq.p, md->nb_ptr.p, md->nb_col.p, md->nb_coloff.p,
                                               md->node_rowlen.p, md->node_rowbase.p, m->rowptr.p, m->colind.p,
                                               m->diagpos.p);
    count_launch(ctx);
    OGB_CUDA(cudaGetLastError());
    OGB_CHECK(pad_matrix_rows(m));
    OGB_CUDA(cudaStreamSynchronize(st));
    OGB_CHECK(check_device_status(ctx, "pattern build"));
    m->has_structure = true;
    m->version++;
    return OGB_OK;
}

int build_loc_pattern(ogb_mtrx *m, int neq, int nelem, const int64_t *loc_ptr_h, const int *loc_h)
{
    ogb_ctx *ctx = m->ctx;
    cudaStream_t st = ctx->stream;
    int64_t nloc = loc_ptr_h[nelem];
    DBuf<int64_t> lptr;
    DBuf<int> loc;
    OGB_CHECK(lptr.alloc(nelem + 1));
    OGB_CHECK(loc.alloc(nloc));
    OGB_CUDA(cudaMemcpyAsync(lptr.p, loc_ptr_h, (nelem + 1) * sizeof(int64_t), cudaMemcpyHostToDevice, st));
    OGB_CUDA(cudaMemcpyAsync(loc.p, loc_h, nloc * sizeof(int), cudaMemcpyHostToDevice, st));
    OGB_CUDA(cudaMemsetAsync(ctx->status.p, 0, sizeof(int), st));
    DBuf<unsigned long long> cnt;
    OGB_CHECK(cnt.alloc(neq + 1));
    OGB_CUDA(cudaMemsetAsync(cnt.p, 0, (neq + 1) * sizeof(unsigned long long), st));
    k_loc_count_inc<<<nblk(nelem), NTHREADS, 0, st>>>(nelem, lptr.p, loc.p, cnt.p);
    DBuf<int64_t> inc_ptr;
    OGB_CHECK(inc_ptr.alloc(neq + 1));
    k_u64_to_i64<<<nblk(neq + 1), NTHREADS, 0, st>>>(neq + 1, cnt.p, inc_ptr.p);
    count_launch(ctx, 2);
    int64_t total = 0;
    OGB_CHECK(exclusive_scan_i64(ctx, inc_ptr.p, inc_ptr.p, neq + 1, &total));
    DBuf<uint32_t> inc;
    DBuf<unsigned int> fill;
    OGB_CHECK(inc.alloc(total));
    OGB_CHECK(fill.alloc(neq));
    OGB_CUDA(cudaMemsetAsync(fill.p, 0, neq * sizeof(unsigned int), st));
    k_loc_fill_inc<<<nblk(nelem), NTHREADS, 0, st>>>(nelem, lptr.p, loc.p, inc_ptr.p, fill.p, inc.p);
    k_sort_segments<uint32_t><<<nblk(neq), NTHREADS, 0, st>>>(neq, inc_ptr.p, inc.p);
    count_launch(ctx, 2);
    DBuf<int64_t> rowcnt;
    OGB_CHECK(rowcnt.alloc(neq + 1));
    OGB_CUDA(cudaMemsetAsync(rowcnt.p + neq, 0, sizeof(int64_t), st));
    k_loc_count_row<<<nblk(neq), NTHREADS, 0, st>>>(neq, lptr.p, loc.p, inc_ptr.p, inc.p, rowcnt.p, ctx->status.p);
    count_launch(ctx);
    int64_t nnz = 0;
    OGB_CHECK(exclusive_scan_i64(ctx, rowcnt.p, rowcnt.p, neq + 1, &nnz));
    OGB_CHECK(check_device_status(ctx, "row pattern"));
    OGB_CHECK(alloc_matrix(m, neq, nnz));
    OGB_CUDA(cudaMemcpyAsync(m->rowptr.p, rowcnt.p, (neq + 1) * sizeof(int64_t), cudaMemcpyDeviceToDevice, st));
    k_loc_fill_row<<<nblk(neq), NTHREADS, 0, st>>>(neq, lptr.p, loc.p, inc_ptr.p, inc.p, m->rowptr.p, m->colind.p,
                                                   m->diagpos.p, ctx->status.p);
    count_launch(ctx);
    OGB_CUDA(cudaGetLastError());
    OGB_CHECK(pad_matrix_rows(m));
    OGB_CUDA(cudaStreamSynchronize(st));
    OGB_CHECK(check_device_status(ctx, "row pattern fill"));
    m->has_structure = true;
    m->version++;
    return OGB_OK;
}

int staged_assemble(ogb_mtrx *m)
{
    ogb_ctx *ctx = m->ctx;
    cudaStream_t st = ctx->stream;
    int nst = (int)m->st_keoff.size();
    if (nst == 0) return OGB_OK;
    DBuf<int64_t> lptr, keoff, cptr, src;
    DBuf<int> loc;
    DBuf<double> ke;
    OGB_CHECK(lptr.alloc(nst + 1));
    OGB_CHECK(keoff.alloc(nst));
    OGB_CHECK(loc.alloc(m->st_loc.size()));
    OGB_CHECK(ke.alloc(m->st_ke.size()));
    OGB_CUDA(cudaMemcpyAsync(lptr.p, m->st_ptr.data(), (nst + 1) * sizeof(int64_t), cudaMemcpyHostToDevice, st));
    OGB_CUDA(cudaMemcpyAsync(keoff.p, m->st_keoff.data(), nst * sizeof(int64_t), cudaMemcpyHostToDevice, st));
    OGB_CUDA(cudaMemcpyAsync(loc.p, m->st_loc.data(), m->st_loc.size() * sizeof(int), cudaMemcpyHostToDevice, st));
    OGB_CUDA(cudaMemcpyAsync(ke.p, m->st_ke.data(), m->st_ke.size() * sizeof(double), cudaMemcpyHostToDevice, st));
    OGB_CUDA(cudaMemsetAsync(ctx->status.p, 0, sizeof(int), st));
    DBuf<unsigned int> cnt;
    OGB_CHECK(cnt.alloc(m->nnz + 1));
    OGB_CUDA(cudaMemsetAsync(cnt.p, 0, (m->nnz + 1) * sizeof(unsigned int), st));
    k_stage_count<<<nst, 64, 0, st>>>(nst, lptr.p, loc.p, m->rowptr.p, m->colind.p, cnt.p, ctx->status.p);
    OGB_CHECK(cptr.alloc(m->nnz + 1));
    k_u64_to_i64<<<nblk(m->nnz + 1), NTHREADS, 0, st>>>(m->nnz + 1, cnt.p, cptr.p);
    count_launch(ctx, 2);
    int64_t total = 0;
    OGB_CHECK(exclusive_scan_i64(ctx, cptr.p, cptr.p, m->nnz + 1, &total));
    OGB_CHECK(check_device_status(ctx, "assemble"));
    OGB_CHECK(src.alloc(total));
    OGB_CUDA(cudaMemsetAsync(cnt.p, 0, (m->nnz + 1) * sizeof(unsigned int), st));
    k_stage_fill<<<nst, 64, 0, st>>>(nst, lptr.p, loc.p, keoff.p, m->rowptr.p, m->colind.p, cptr.p, cnt.p, src.p);
    k_sort_segments<int64_t><<<nblk(m->nnz), NTHREADS, 0, st>>>(m->nnz, cptr.p, src.p);
    k_stage_apply<<<nblk(m->nnz), NTHREADS, 0, st>>>(m->nnz, cptr.p, src.p, ke.p, m->val.p);
    count_launch(ctx, 3);
    OGB_CUDA(cudaGetLastError());
    OGB_CUDA(cudaStreamSynchronize(st));
    m->st_ptr.assign(1, 0);
    m->st_loc.clear();
    m->st_keoff.clear();
    m->st_ke.clear();
    m->version++;
    return OGB_OK;
}

}  // namespace ogb

// ---------------------------------------------------------------------------
// Node-block SELL-32 copy of a model-built matrix (solver storage).
namespace ogb {
namespace {

__global__ void k_act_flags(int nnodes, int ndofpn, const int *eq, int64_t *flag)
{
    int A = blockIdx.x * blockDim.x + threadIdx.x;
    if (A > nnodes) return;
    flag[A] = A < nnodes ? (nfree_of(eq, ndofpn, A) > 0) : 0;
}

// Node-space row of every active node: its rank among the active nodes of its
// instance plus the instance's row base (instances start on 1024-row boundaries).
__global__ void k_act_index(int nnodes, int ndofpn, const int *eq, const int64_t *scan, int ninst,
                            const int *inst_start, const int64_t *inst_rank0, const int64_t *inst_base, int *act,
                            int *rownode)
{
    int A = blockIdx.x * blockDim.x + threadIdx.x;
    if (A >= nnodes) return;
    if (nfree_of(eq, ndofpn, A) > 0) {
        int lo = 0, hi = ninst - 1;
        while (lo < hi) {   // last instance whose first node is <= A
            int mid = (lo + hi + 1) >> 1;
            if (inst_start[mid] <= A) lo = mid; else hi = mid - 1;
        }
        int a = (int)(scan[A] - inst_rank0[lo] + inst_base[lo]);
        act[A] = a;
        rownode[a] = A;
    } else {
        act[A] = -1;
    }
}

// Width (active neighbours) of every row; padding rows (rownode < 0) get one
// identity block.
__global__ void k_row_width(int nrows_pad, int nact, const int *rownode, const int64_t *nb_ptr, const int *nb_col,
                            const int *act, int *width)
{
    int a = blockIdx.x * blockDim.x + threadIdx.x;
    if (a >= nrows_pad) return;
    if (rownode[a] < 0) {
        width[a] = 1;
        return;
    }
    int A = rownode[a], w = 0;
    for (int64_t k = nb_ptr[A]; k < nb_ptr[A + 1]; ++k) w += act[nb_col[k]] >= 0;
    width[a] = w;
}

__global__ void k_slice_width(int nslices, const int *width, int *sl_width, int64_t *slots)
{
    int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s > nslices) return;
    if (s == nslices) {
        slots[s] = 0;
        return;
    }
    int w = 0;
    for (int r = 0; r < 32; ++r) w = max(w, width[s * 32 + r]);
    sl_width[s] = w;
    slots[s] = (int64_t)w * 32;
}

template <int ND>
__global__ void k_fill_sell(int nrows_pad, int nact, const int *rownode, const int64_t *nb_ptr, const int *nb_col,
                            const int *act, const int64_t *sl_ptr, const int *sl_width, int *col, int64_t *diag,
                            int64_t *blk_slot, double *v64, float *v32)
{
    int a = blockIdx.x * blockDim.x + threadIdx.x;
    if (a >= nrows_pad) return;
    int s = a >> 5, r = a & 31;
    int64_t base = sl_ptr[s];
    int w = sl_width[s];
    int kk = 0;
    if (rownode[a] >= 0) {
        int A = rownode[a];
        for (int64_t k = nb_ptr[A]; k < nb_ptr[A + 1]; ++k) {
            int B = nb_col[k];
            int b = act[B];
            if (b < 0) {
                blk_slot[k] = -1;
                continue;
            }
            int64_t slot = base + (int64_t)kk * 32 + r;
            col[slot] = b;
            blk_slot[k] = slot;
            if (B == A) diag[a] = slot;
            ++kk;
        }
    } else {
        int64_t slot = base + r;   // identity block
        col[slot] = a;
        diag[a] = slot;
        for (int e = 0; e < ND * ND; ++e) {
            double v = (e % (ND + 1) == 0) ? 1.0 : 0.0;
            v64[(slot - r) * ND * ND + 32 * e + r] = v;
            v32[(slot - r) * ND * ND + 32 * e + r] = (float)v;
        }
        kk = 1;
    }
    for (; kk < w; ++kk) col[base + (int64_t)kk * 32 + r] = a < nact ? a : a;   // zero-valued padding slots
}

__global__ void k_ns_of_eq(int nnodes, int ndofpn, const int *eq, const int *act, int *ns_of_eq)
{
    int A = blockIdx.x * blockDim.x + threadIdx.x;
    if (A >= nnodes || act[A] < 0) return;
    for (int d = 0; d < ndofpn; ++d) {
        int q = eq[(size_t)A * ndofpn + d];
        if (q > 0) ns_of_eq[q - 1] = act[A] * ndofpn + d;
    }
}

}  // namespace

int build_sell(ogb_model *md, ogb_mtrx *m)
{
    ogb_ctx *ctx = md->ctx;
    cudaStream_t st = ctx->stream;
    const int nn = md->nnodes, nd = md->ndofpn;
    SellMat &S = m->sell;
    S.nd = nd;
    S.group[0] = S.group[1] = 0;   // the SpMV autotuner runs again for the new structure
    S.bform32 = 0;
    S.half.reset();                 // and the half-stored copy is rebuilt on first use
    DBuf<int64_t> flag;
    OGB_CHECK(flag.alloc(nn + 1));
    k_act_flags<<<nblk(nn + 1), NTHREADS, 0, st>>>(nn, nd, md->eq.p, flag.p);
    count_launch(ctx);
    int64_t nact = 0;
    OGB_CHECK(exclusive_scan_i64(ctx, flag.p, flag.p, nn + 1, &nact));
    S.nact = (int)nact;
    // instances (independent meshes of a batch): each starts on a 1024-row boundary
    // of node space, so every reduction unit of the solver belongs to one instance
    const int ninst = (int)md->inst_start.size() - 1;
    std::vector<int64_t> rank(nn + 1);
    OGB_CUDA(cudaMemcpyAsync(rank.data(), flag.p, (nn + 1) * sizeof(int64_t), cudaMemcpyDeviceToHost, st));
    OGB_CUDA(cudaStreamSynchronize(st));
    std::vector<int64_t> rank0(ninst), base(ninst + 1, 0);
    S.inst_row_base.assign(ninst + 1, 0);
    for (int i = 0; i < ninst; ++i) {
        rank0[i] = rank[md->inst_start[i]];
        int64_t na = rank[md->inst_start[i + 1]] - rank0[i];
        base[i + 1] = base[i] + ceil_div(na > 0 ? na : 1, INST_ALIGN) * INST_ALIGN;
    }
    S.inst_row_base = base;
    S.ninst = ninst;
    const int nslices = (int)(base[ninst] / 32);
    S.nslices = nslices;
    const int nrows_pad = nslices * 32;
    DBuf<int> rownode, width, d_start;
    DBuf<int64_t> d_rank0, d_base;
    OGB_CHECK(md->act.alloc(nn));
    OGB_CHECK(rownode.alloc(nrows_pad));
    OGB_CHECK(width.alloc(nrows_pad));
    OGB_CHECK(d_start.alloc(ninst + 1));
    OGB_CHECK(d_rank0.alloc(ninst));
    OGB_CHECK(d_base.alloc(ninst + 1));
    OGB_CUDA(cudaMemcpyAsync(d_start.p, md->inst_start.data(), (ninst + 1) * sizeof(int), cudaMemcpyHostToDevice, st));
    OGB_CUDA(cudaMemcpyAsync(d_rank0.p, rank0.data(), ninst * sizeof(int64_t), cudaMemcpyHostToDevice, st));
    OGB_CUDA(cudaMemcpyAsync(d_base.p, base.data(), (ninst + 1) * sizeof(int64_t), cudaMemcpyHostToDevice, st));
    OGB_CUDA(cudaMemsetAsync(rownode.p, 0xff, nrows_pad * sizeof(int), st));   // -1: padding row
    k_act_index<<<nblk(nn), NTHREADS, 0, st>>>(nn, nd, md->eq.p, flag.p, ninst, d_start.p, d_rank0.p, d_base.p,
                                               md->act.p, rownode.p);
    k_row_width<<<nblk(nrows_pad), NTHREADS, 0, st>>>(nrows_pad, S.nact, rownode.p, md->nb_ptr.p, md->nb_col.p,
                                                      md->act.p, width.p);
    OGB_CHECK(S.sl_ptr.alloc(nslices + 1));
    OGB_CHECK(S.sl_width.alloc(nslices));
    k_slice_width<<<nblk(nslices + 1), NTHREADS, 0, st>>>(nslices, width.p, S.sl_width.p, S.sl_ptr.p);
    count_launch(ctx, 3);
    int64_t nslots = 0;
    OGB_CHECK(exclusive_scan_i64(ctx, S.sl_ptr.p, S.sl_ptr.p, nslices + 1, &nslots));
    S.nslots = nslots;
    OGB_CHECK(S.col.alloc(nslots));
    OGB_CHECK(S.diag.alloc(nrows_pad));
    OGB_CHECK(S.v64.alloc((size_t)nslots * nd * nd));
    OGB_CHECK(S.v32.alloc((size_t)nslots * nd * nd));
    OGB_CHECK(md->blk_slot.alloc(md->nblocks > 0 ? md->nblocks : 1));
    OGB_CUDA(cudaMemsetAsync(S.v64.p, 0, (size_t)nslots * nd * nd * sizeof(double), st));
    OGB_CUDA(cudaMemsetAsync(S.v32.p, 0, (size_t)nslots * nd * nd * sizeof(float), st));
    if (nd == 3)
        k_fill_sell<3><<<nblk(nrows_pad), NTHREADS, 0, st>>>(nrows_pad, S.nact, rownode.p, md->nb_ptr.p, md->nb_col.p,
                                                             md->act.p, S.sl_ptr.p, S.sl_width.p, S.col.p, S.diag.p,
                                                             md->blk_slot.p, S.v64.p, S.v32.p);
    else
        k_fill_sell<2><<<nblk(nrows_pad), NTHREADS, 0, st>>>(nrows_pad, S.nact, rownode.p, md->nb_ptr.p, md->nb_col.p,
                                                             md->act.p, S.sl_ptr.p, S.sl_width.p, S.col.p, S.diag.p,
                                                             md->blk_slot.p, S.v64.p, S.v32.p);
    OGB_CHECK(S.ns_of_eq.alloc(md->neq > 0 ? md->neq : 1));
    k_ns_of_eq<<<nblk(nn), NTHREADS, 0, st>>>(nn, nd, md->eq.p, md->act.p, S.ns_of_eq.p);
    count_launch(ctx, 2);
    OGB_CUDA(cudaGetLastError());
    OGB_CUDA(cudaStreamSynchronize(st));   // the temporaries above are freed on return
    S.v32_version = -1;
    m->has_sell = true;
    return OGB_OK;
}

}  // namespace ogb
