// Incomplete-Cholesky preconditioner of the IML solver (lsprecond 4,
// CompCol_ICPreconditioner, src/core/iml/icprecond.C:40-226).
//
// Factorization (host, once per matrix version, as the reference does it on
// its host): the lower triangle of the symmetric matrix by columns -- column k
// holds rows >= k, the diagonal first; for the symmetric pattern stored here
// that is row k of the CSR restricted to columns >= k -- then the reference's
// ICFactor loop (icprecond.C:133-163) kept step for step: the diagonal takes a
// square root, the column is divided by it, and the columns of the rows below
// are updated by the same nested search over row indices. That search only
// matches at the last entry of column k (its successor test reads into the next
// column), so the factor it produces is not a textbook IC(0); parity requires
// the same loop, not a cleaner one.
//
// Application (device): ICSolve (icprecond.C:166-190) is a forward solve by
// columns and a backward solve by columns. On the device both run by rows,
// level by level: row i's forward value needs the rows c < i of its transposed
// column entries, its backward value the rows r > i of its own column. Each
// solve is one launch of one thread-block cluster that steps through the levels
// with the cluster barrier between them (rows of a level spread over the
// cluster's SMs, a thread per row, each row's entries loaded in chunks before
// their differences). The products are accumulated in
// the reference's order (columns resp. rows ascending, starting from zero) with
// separate rounded multiply and subtract, so z = M^-1 r is bitwise the
// reference's.
//
// lsprecond 2 (CompCol_ILUPreconditioner, src/core/iml/iluprecond.C:75-193,
// 265-289) is built the same way: the matrix split by columns into a strictly
// lower L (unit diagonal implied) and an upper U with the diagonal last, the
// reference's factorization loop, and its solves L w = x (columns ascending,
// each row's sum started from zero and x added last) and U y = w (columns
// descending, each row's sum started from w).
#include <math.h>

#include <algorithm>
#include <vector>

#include "internal.cuh"

namespace ogb {

namespace {

// Row i of a level of one triangular solve, in the reference's arithmetic
// (separately rounded products and differences, entries in stored order):
//   IC  (KIND 4): out_i = (in_i + sum(-v_e out_c)) / d_i, forward and backward;
//   ILU (KIND 2): forward out_i = sum(-v_e out_c) + in_i, backward
//                 out_i = (in_i - v_e out_c - ...) / d_i.
template <int KIND, bool FWD, bool L2 = false>
__device__ __forceinline__ void tri_row(int i, const int64_t *__restrict__ ptr, const int *__restrict__ col,
                                        const double *__restrict__ val, const double *__restrict__ diag,
                                        const double *__restrict__ in, double *out)
{
    // L2: out[] is written by other SMs in this launch, so it is read from L2
    auto rd = [&](int c) { return L2 ? __ldcg(out + c) : out[c]; };
    double acc = (KIND == 2 && !FWD) ? in[i] : 0.0;
    // the entries of a chunk are loaded before the chunk's differences, which
    // keep the stored order
    constexpr int CH = 16;
    int64_t e = ptr[i];
    const int64_t e1 = ptr[i + 1];
    for (; e + CH <= e1; e += CH) {
        int cc[CH];
        double vv[CH], oo[CH];
#pragma unroll
        for (int k = 0; k < CH; ++k) {
            cc[k] = col[e + k];
            vv[k] = val[e + k];
        }
#pragma unroll
        for (int k = 0; k < CH; ++k) oo[k] = rd(cc[k]);
#pragma unroll
        for (int k = 0; k < CH; ++k) acc = __dsub_rn(acc, __dmul_rn(vv[k], oo[k]));
    }
    for (; e < e1; ++e) acc = __dsub_rn(acc, __dmul_rn(val[e], rd(col[e])));
    if (KIND == 4) out[i] = __ddiv_rn(__dadd_rn(in[i], acc), diag[i]);
    else if (FWD) out[i] = __dadd_rn(acc, in[i]);
    else out[i] = __ddiv_rn(acc, diag[i]);
}

// Every level of one triangular solve in one launch of one thread-block
// cluster (TRI_CLUSTER CTAs on as many SMs): the rows of a level go round-robin
// over the CTAs first (the narrow FP64 pipes of several SMs share the work), a
// thread per row, and the cluster's hardware barrier (release / acquire at
// cluster scope) separates the levels; out[] is read from L2, where the other
// SMs' stores of the previous levels are. What a row needs besides out[] (its
// index, entry range, first TRI_PRE columns and values, in_i, d_i) is loaded
// before the barrier that precedes its level, so after the barrier a row costs
// one round of out[] loads and its chain of differences.
constexpr int TRI_THREADS = 256;
constexpr int TRI_CLUSTER = 8;
constexpr int TRI_PRE = 40;
template <int KIND, bool FWD>
__global__ void __launch_bounds__(TRI_THREADS) k_tri_cluster(int nlev, const int *__restrict__ lev,
                                                             const int *__restrict__ rows,
                                                             const int64_t *__restrict__ ptr,
                                                             const int *__restrict__ col,
                                                             const double *__restrict__ val,
                                                             const double *__restrict__ diag,
                                                             const double *__restrict__ in, double *out,
                                                             const PcgScal *sc)
{
    if (sc && (sc->done || sc->reliable)) return;   // the same for every CTA of the cluster
    const int stride = TRI_CLUSTER * TRI_THREADS, q0 = threadIdx.x * TRI_CLUSTER + (int)blockIdx.x;
    int row = -1;
    int64_t e0 = 0, e1 = 0;
    int cc[TRI_PRE];
    double vv[TRI_PRE];
    double xin = 0.0, dg = 1.0;
    auto fetch = [&](int l) {
        row = -1;
        if (l >= nlev) return;
        const int r0 = lev[l], w = lev[l + 1] - r0;
        if (q0 >= w) return;
        row = rows[r0 + q0];
        e0 = ptr[row];
        e1 = ptr[row + 1];
#pragma unroll
        for (int k = 0; k < TRI_PRE; ++k) {
            cc[k] = e0 + k < e1 ? col[e0 + k] : 0;
            vv[k] = e0 + k < e1 ? val[e0 + k] : 0.0;
        }
        xin = in[row];
        dg = (KIND == 4 || !FWD) ? diag[row] : 1.0;
    };
    fetch(0);
    for (int l = 0; l < nlev; ++l) {
        if (row >= 0) {
            double acc = (KIND == 2 && !FWD) ? xin : 0.0;
            const int n = (int)min(e1 - e0, (int64_t)TRI_PRE);
            double oo[TRI_PRE];
#pragma unroll
            for (int k = 0; k < TRI_PRE; ++k) oo[k] = k < n ? __ldcg(out + cc[k]) : 0.0;
#pragma unroll
            for (int k = 0; k < TRI_PRE; ++k)
                if (k < n) acc = __dsub_rn(acc, __dmul_rn(vv[k], oo[k]));
            for (int64_t e = e0 + TRI_PRE; e < e1; ++e) acc = __dsub_rn(acc, __dmul_rn(val[e], __ldcg(out + col[e])));
            if (KIND == 4) out[row] = __ddiv_rn(__dadd_rn(xin, acc), dg);
            else if (FWD) out[row] = __dadd_rn(acc, xin);
            else out[row] = __ddiv_rn(acc, dg);
        }
        // rows of a level wider than the cluster's threads
        const int r0 = lev[l], w = lev[l + 1] - r0;
        for (int q = q0 + stride; q < w; q += stride) tri_row<KIND, FWD, true>(rows[r0 + q], ptr, col, val, diag, in, out);
        fetch(l + 1);
        asm volatile("barrier.cluster.arrive.release.aligned;\n"
                     "barrier.cluster.wait.acquire.aligned;\n" ::: "memory");
    }
}

// Rows grouped by level (counting sort, rows ascending within a level).
void group_levels(const std::vector<int> &lev, int nlev, std::vector<int> &rows, std::vector<int> &start)
{
    start.assign(nlev + 1, 0);
    for (int l : lev) start[l + 1]++;
    for (int l = 0; l < nlev; ++l) start[l + 1] += start[l];
    rows.assign(lev.size(), 0);
    std::vector<int> fill(start.begin(), start.end() - 1);
    for (int i = 0; i < (int)lev.size(); ++i) rows[fill[lev[i]]++] = i;
}

}  // namespace

namespace {

// Device copy of a factor given by its forward / backward rows and diagonal.
int upload_factor(ogb_mtrx *m, int kind, const std::vector<int64_t> &fp, const std::vector<int> &fc,
                  const std::vector<double> &fv, const std::vector<int64_t> &bp, const std::vector<int> &bc,
                  const std::vector<double> &bv, const std::vector<double> &dg)
{
    IcFactor &F = m->ic;
    cudaStream_t s = m->ctx->stream;
    const int n = (int)dg.size();
    std::vector<int> lf(n, 0), lb(n, 0);
    int nlf = 0, nlb = 0;
    for (int i = 0; i < n; ++i) {
        int l = 0;
        for (int64_t e = fp[i]; e < fp[i + 1]; ++e) l = std::max(l, lf[fc[e]] + 1);
        lf[i] = l;
        nlf = std::max(nlf, l + 1);
    }
    for (int i = n - 1; i >= 0; --i) {
        int l = 0;
        for (int64_t e = bp[i]; e < bp[i + 1]; ++e) l = std::max(l, lb[bc[e]] + 1);
        lb[i] = l;
        nlb = std::max(nlb, l + 1);
    }
    std::vector<int> frows, brows;
    group_levels(lf, nlf, frows, F.flev);
    group_levels(lb, nlb, brows, F.blev);
    auto up = [&](auto &dst, const auto &src) -> int {
        using T = typename std::decay_t<decltype(src)>::value_type;
        OGB_CHECK(dst.alloc(src.empty() ? 1 : src.size()));
        if (!src.empty())
            OGB_CUDA(cudaMemcpyAsync(dst.p, src.data(), src.size() * sizeof(T), cudaMemcpyHostToDevice, s));
        return OGB_OK;
    };
    OGB_CHECK(up(F.fptr, fp));
    OGB_CHECK(up(F.fcol, fc));
    OGB_CHECK(up(F.fval, fv));
    OGB_CHECK(up(F.bptr, bp));
    OGB_CHECK(up(F.bcol, bc));
    OGB_CHECK(up(F.bval, bv));
    OGB_CHECK(up(F.diag, dg));
    OGB_CHECK(up(F.frows, frows));
    OGB_CHECK(up(F.brows, brows));
    OGB_CHECK(up(F.d_flev, F.flev));
    OGB_CHECK(up(F.d_blev, F.blev));
    OGB_CHECK(F.work.alloc(n > 0 ? n : 1));
    OGB_CUDA(cudaStreamSynchronize(s));   // the host arrays are freed on return
    F.n = n;
    F.kind = kind;
    F.version = m->version;
    return OGB_OK;
}

// The matrix by rows on the host (npad rows, identity padding included).
int host_csr(ogb_mtrx *m, std::vector<int64_t> &rp, std::vector<int> &ci, std::vector<double> &va)
{
    cudaStream_t s = m->ctx->stream;
    const int n = m->npad;
    const int64_t ntot = m->nnz + (m->npad - m->neq);
    rp.resize(n + 1);
    ci.resize(ntot);
    va.resize(ntot);
    OGB_CUDA(cudaMemcpyAsync(rp.data(), m->rowptr.p, (n + 1) * sizeof(int64_t), cudaMemcpyDeviceToHost, s));
    OGB_CUDA(cudaMemcpyAsync(ci.data(), m->colind.p, ntot * sizeof(int), cudaMemcpyDeviceToHost, s));
    OGB_CUDA(cudaMemcpyAsync(va.data(), m->val.p, ntot * sizeof(double), cudaMemcpyDeviceToHost, s));
    OGB_CUDA(cudaStreamSynchronize(s));
    return OGB_OK;
}

int build_ilu(ogb_mtrx *m)
{
    std::vector<int64_t> rp;
    std::vector<int> ci;
    std::vector<double> va;
    OGB_CHECK(host_csr(m, rp, ci, va));
    const int n = m->npad;
    // column i of the (symmetric) matrix = row i: L takes rows > i, U rows <= i
    // (CompCol_ILUPreconditioner::initialize, iluprecond.C:75-130)
    std::vector<int> lp(n + 1, 0), up_(n + 1, 0);
    for (int i = 0; i < n; ++i) {
        int l = 0, u = 0;
        for (int64_t j = rp[i]; j < rp[i + 1]; ++j) (ci[j] > i ? l : u) += 1;
        lp[i + 1] = lp[i] + l;
        up_[i + 1] = up_[i] + u;
    }
    std::vector<int> lr(lp[n]), ur(up_[n]);
    std::vector<double> lv(lp[n]), uv(up_[n]);
    for (int i = 0; i < n; ++i) {
        int a = lp[i], b = up_[i];
        for (int64_t j = rp[i]; j < rp[i + 1]; ++j) {
            if (ci[j] > i) {
                lr[a] = ci[j];
                lv[a++] = va[j];
            } else {
                ur[b] = ci[j];
                uv[b++] = va[j];
            }
        }
        if (up_[i + 1] == up_[i] || ur[up_[i + 1] - 1] != i)
            return fail(OGB_E_ZERODIAG, "ILU preconditioner: diagonal not found");
    }
    // the factorization loop (iluprecond.C:134-167)
    for (int i = 0; i < n - 1; ++i) {
        double multiplier = uv[up_[i + 1] - 1];
        for (int j = lp[i]; j < lp[i + 1]; ++j) lv[j] /= multiplier;
        for (int j = up_[i + 1]; j < up_[i + 2] - 1; ++j) {
            multiplier = uv[j];
            int qn = j + 1, rn = lp[i + 1], pn;
            for (pn = lp[ur[j]]; pn < lp[ur[j] + 1] && lr[pn] <= i + 1; ++pn) {
                while (qn < up_[i + 2] && ur[qn] < lr[pn]) ++qn;
                if (qn < up_[i + 2] && lr[pn] == ur[qn]) uv[qn] -= multiplier * lv[pn];
            }
            for (; pn < lp[ur[j] + 1]; ++pn) {
                while (rn < lp[i + 2] && lr[rn] < lr[pn]) ++rn;
                if (rn < lp[i + 2] && lr[pn] == lr[rn]) lv[rn] -= multiplier * lv[pn];
            }
        }
    }
    // forward rows: (c, L_ic) from the columns c < i, c ascending
    std::vector<int64_t> fp(n + 1, 0);
    for (int c = 0; c < n; ++c)
        for (int t = lp[c]; t < lp[c + 1]; ++t) fp[lr[t] + 1]++;
    for (int i = 0; i < n; ++i) fp[i + 1] += fp[i];
    std::vector<int> fc(fp[n]);
    std::vector<double> fv(fp[n]);
    {
        std::vector<int64_t> fill(fp.begin(), fp.end() - 1);
        for (int c = 0; c < n; ++c)
            for (int t = lp[c]; t < lp[c + 1]; ++t) {
                const int64_t e = fill[lr[t]]++;
                fc[e] = c;
                fv[e] = lv[t];
            }
    }
    // backward rows: (c, U_rc) from the columns c > r, c descending; the diagonal
    std::vector<int64_t> bp(n + 1, 0);
    for (int c = 0; c < n; ++c)
        for (int t = up_[c]; t < up_[c + 1] - 1; ++t) bp[ur[t] + 1]++;
    for (int i = 0; i < n; ++i) bp[i + 1] += bp[i];
    std::vector<int> bc(bp[n]);
    std::vector<double> bv(bp[n]), dg(n);
    {
        std::vector<int64_t> fill(bp.begin(), bp.end() - 1);
        for (int c = n - 1; c >= 0; --c) {
            dg[c] = uv[up_[c + 1] - 1];
            for (int t = up_[c]; t < up_[c + 1] - 1; ++t) {
                const int64_t e = fill[ur[t]]++;
                bc[e] = c;
                bv[e] = uv[t];
            }
        }
    }
    return upload_factor(m, 2, fp, fc, fv, bp, bc, bv, dg);
}

}  // namespace

int build_ic(ogb_mtrx *m)
{
    IcFactor &F = m->ic;
    if (F.version == m->version && F.kind == m->precond) return OGB_OK;
    if (m->precond == 2) return build_ilu(m);
    const int n = m->npad;
    std::vector<int64_t> rp;
    std::vector<int> ci;
    std::vector<double> va;
    OGB_CHECK(host_csr(m, rp, ci, va));
    // lower triangle by columns (CompCol_ICPreconditioner::initialize, icprecond.C:64-107)
    std::vector<int> pntr(n + 1, 0);
    for (int k = 0; k < n; ++k) {
        int c = 0;
        for (int64_t j = rp[k]; j < rp[k + 1]; ++j) c += ci[j] >= k;
        pntr[k + 1] = pntr[k] + c;
    }
    const int nz = pntr[n];
    std::vector<int> indx(nz);
    std::vector<double> val(nz);
    for (int k = 0; k < n; ++k) {
        int t = pntr[k];
        for (int64_t j = rp[k]; j < rp[k + 1]; ++j)
            if (ci[j] >= k) {
                indx[t] = ci[j];
                val[t] = va[j];
                ++t;
            }
        if (pntr[k] == pntr[k + 1] || indx[pntr[k]] != k) return fail(OGB_E_ZERODIAG, "IC preconditioner: diagonal not found");
    }
    // ICFactor (icprecond.C:133-163), the same loop nest. indx gets one sentinel
    // entry: the successor test of the last entry of the last column reads one
    // past the end there.
    indx.push_back(n);
    for (int k = 0; k < n - 1; ++k) {
        const int d = pntr[k];
        const double z = val[d] = sqrt(val[d]);
        for (int i = d + 1; i < pntr[k + 1]; ++i) val[i] /= z;
        for (int i = d + 1; i < pntr[k + 1]; ++i) {
            const double zi = val[i];
            const int h = indx[i];
            int g = i;
            for (int j = pntr[h]; j < pntr[h + 1]; ++j)
                for (; g < pntr[k + 1] && indx[g + 1] <= indx[j]; ++g)
                    if (indx[g] == indx[j]) val[j] -= zi * val[g];
        }
    }
    if (n > 0) val[pntr[n - 1]] = sqrt(val[pntr[n - 1]]);
    indx.pop_back();
    // forward rows: entries (c, L_ic) from the columns c < i, c ascending
    std::vector<int64_t> fp(n + 1, 0);
    for (int c = 0; c < n; ++c)
        for (int t = pntr[c] + 1; t < pntr[c + 1]; ++t) fp[indx[t] + 1]++;
    for (int i = 0; i < n; ++i) fp[i + 1] += fp[i];
    std::vector<int> fc(fp[n]);
    std::vector<double> fv(fp[n]);
    {
        std::vector<int64_t> fill(fp.begin(), fp.end() - 1);
        for (int c = 0; c < n; ++c)
            for (int t = pntr[c] + 1; t < pntr[c + 1]; ++t) {
                const int64_t e = fill[indx[t]]++;
                fc[e] = c;
                fv[e] = val[t];
            }
    }
    // backward rows: row i's own column below the diagonal, rows ascending
    std::vector<int64_t> bp(n + 1, 0);
    for (int i = 0; i < n; ++i) bp[i + 1] = bp[i] + (pntr[i + 1] - pntr[i] - 1);
    std::vector<int> bc(bp[n]);
    std::vector<double> bv(bp[n]), dg(n);
    for (int i = 0; i < n; ++i) {
        dg[i] = val[pntr[i]];
        for (int t = pntr[i] + 1; t < pntr[i + 1]; ++t) {
            bc[bp[i] + (t - pntr[i] - 1)] = indx[t];
            bv[bp[i] + (t - pntr[i] - 1)] = val[t];
        }
    }
    return upload_factor(m, 4, fp, fc, fv, bp, bc, bv, dg);
}

template <int KIND, bool FWD>
int tri_solve(cudaStream_t s, const IcFactor &F, bool fwd_data, const double *in, double *out, const PcgScal *sc)
{
    const std::vector<int> &lev = fwd_data ? F.flev : F.blev;
    const int nlev = (int)lev.size() - 1;
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(TRI_CLUSTER);
    cfg.blockDim = dim3(TRI_THREADS);
    cfg.stream = s;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = TRI_CLUSTER;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    OGB_CUDA(cudaLaunchKernelEx(&cfg, k_tri_cluster<KIND, FWD>, nlev, (const int *)(fwd_data ? F.d_flev.p : F.d_blev.p),
                                (const int *)(fwd_data ? F.frows.p : F.brows.p),
                                (const int64_t *)(fwd_data ? F.fptr.p : F.bptr.p),
                                (const int *)(fwd_data ? F.fcol.p : F.bcol.p),
                                (const double *)(fwd_data ? F.fval.p : F.bval.p), (const double *)F.diag.p, in, out,
                                sc));
    return OGB_OK;
}

int launch_ic_solve(ogb_mtrx *m, const double *r, double *z, const PcgScal *sc)
{
    IcFactor &F = m->ic;
    cudaStream_t s = m->ctx->stream;
    if (F.kind == 2) {
        OGB_CHECK((tri_solve<2, true>(s, F, true, r, F.work.p, sc)));
        OGB_CHECK((tri_solve<2, false>(s, F, false, F.work.p, z, sc)));
    } else {
        OGB_CHECK((tri_solve<4, true>(s, F, true, r, F.work.p, sc)));
        OGB_CHECK((tri_solve<4, false>(s, F, false, F.work.p, z, sc)));
    }
    count_launch(m->ctx, 2);
    OGB_CUDA(cudaGetLastError());
    return OGB_OK;
}

}  // namespace ogb
