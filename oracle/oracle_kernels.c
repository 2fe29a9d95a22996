/*
 * ORACLE — CPU restatement of the reference's sampled-ALS hot path
 * (vbharadwaj-bk/rdist_tensor, exafac/cpp_ext).  TEST INFRASTRUCTURE ONLY:
 * tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg may load it,
 * as the checker or as the timed CPU port; the product never does.
 *
 * Parity pin: the golden fixtures under tests/golden/, generated from the reference itself compiled
 * here (oracle/build_ref.sh, tests/golden/make_golden.py).
 *
 * This file holds the loops; oracle/oracle.py holds the dense R x R algebra and
 * the step orchestration.  Every function names the reference lines it follows.
 * Built by oracle/Makefile into oracle/_build/liboracle.so (gcc -O2 -fopenmp;
 * no fast-math, so sequential sums keep the reference's order).
 */
#include <math.h>
#include <omp.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

/* ------------------------------------------------------------------------- */
/* PartitionTree shape (partition_tree.hpp:82-115; common.h:677-693)         */
/* ------------------------------------------------------------------------- */
typedef struct {
    int64_t n, F, R;
    int64_t leaf_count, node_count;
    int64_t lfill_level, lfill_count;
    int64_t nodes_upto_lfill, nodes_before_lfill, complete_level_offset;
} or_tree_t;

void or_tree_shape(int64_t n, int64_t F, int64_t R, or_tree_t* t) {
    t->n = n;
    t->F = F;
    t->R = R;
    t->leaf_count = (n + F - 1) / F;
    t->node_count = 2 * t->leaf_count - 1;
    t->lfill_level = 0;
    t->lfill_count = 1;
    while (t->lfill_count * 2 <= t->leaf_count) {
        t->lfill_level++;
        t->lfill_count *= 2;
    }
    t->nodes_upto_lfill = t->lfill_count * 2 - 1;
    t->nodes_before_lfill = t->lfill_count - 1;
    int64_t div2 = (t->node_count - t->nodes_upto_lfill) / 2;
    t->complete_level_offset = t->nodes_before_lfill - div2;
}

static inline int64_t tree_leaf_idx(const or_tree_t* t, int64_t c) {
    return c >= t->nodes_upto_lfill ? c - t->nodes_upto_lfill : c - t->complete_level_offset;
}
static inline int tree_is_leaf(const or_tree_t* t, int64_t c) { return 2 * c + 1 >= t->node_count; }

/* build_tree (partition_tree.hpp:117-167): leaf Gram = U_blk^T U_blk over the
 * F rows of the leaf (fewer for the last leaf), then bottom-up pairwise sums
 * level by level.  G holds full symmetric R x R blocks. */
void or_tree_build(const or_tree_t* t, const double* U, double* G) {
    const int64_t R = t->R, R2 = R * R, F = t->F;
    const int64_t first_leaf = t->node_count - t->leaf_count;
    memset(G, 0, sizeof(double) * (size_t)(t->node_count * R2));
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < t->leaf_count; i++) {
        int64_t leaf = tree_leaf_idx(t, first_leaf + i);
        int64_t rows = F < (t->n - leaf * F) ? F : (t->n - leaf * F);
        double* g = G + (first_leaf + i) * R2;
        for (int64_t r = 0; r < rows; r++) {
            const double* u = U + (leaf * F + r) * R;
            for (int64_t a = 0; a < R; a++)
                for (int64_t b = a; b < R; b++) g[a * R + b] += u[a] * u[b];
        }
        for (int64_t a = 0; a < R; a++)
            for (int64_t b = 0; b < a; b++) g[a * R + b] = g[b * R + a];
    }
    int64_t start = t->nodes_before_lfill, end = first_leaf;
    for (int64_t lvl = t->lfill_level; lvl >= 0; lvl--) {
#pragma omp parallel for schedule(static)
        for (int64_t c = start; c < end; c++)
            for (int64_t j = 0; j < R2; j++) G[c * R2 + j] += G[(2 * c + 1) * R2 + j] + G[(2 * c + 2) * R2 + j];
        end = start;
        start = ((start + 1) / 2) - 1;
    }
}

/* Elementwise multiply of every node by a fixed R x R matrix
 * (multiply_matrices_against_provided, partition_tree.hpp:176-187). */
void or_tree_hadamard(const or_tree_t* t, double* G, const double* M) {
    const int64_t R2 = t->R * t->R;
#pragma omp parallel for schedule(static)
    for (int64_t c = 0; c < t->node_count; c++)
        for (int64_t j = 0; j < R2; j++) G[c * R2 + j] *= M[j];
}

static inline double quad_form(const double* g, const double* x, int64_t R) {
    /* x^T G x as dsymv (y = G x) followed by a dot product. */
    double acc = 0.0;
    for (int64_t a = 0; a < R; a++) {
        double y = 0.0;
        for (int64_t b = 0; b < R; b++) y += g[a * R + b] * x[b];
        acc += x[a] * y;
    }
    return acc;
}

/* PTSample (partition_tree.hpp:204-380) for J samples: descent driven by x
 * (the reference's scaled_h), explicit draws; the chosen row is written to
 * out_idx and hmul[i] *= U[row] (the reference's h). */
void or_tree_sample(const or_tree_t* t, const double* G, const double* U, int64_t J, const double* x, double* hmul,
                    const double* draws, uint32_t* out_idx) {
    const int64_t R = t->R, R2 = R * R, F = t->F;
#pragma omp parallel
    {
        double* q = (double*)malloc(sizeof(double) * (size_t)F);
#pragma omp for schedule(static)
        for (int64_t i = 0; i < J; i++) {
            const double* xi = x + i * R;
            double d = draws[i];
            int64_t c = 0;
            double low = 0.0, high = 1.0;
            double m = quad_form(G, xi, R);
            for (int64_t lvl = 0; lvl < t->lfill_level; lvl++) {
                double mL = quad_form(G + (2 * c + 1) * R2, xi, R);
                double cutoff = low + mL / m;
                if (d <= cutoff) {
                    c = 2 * c + 1;
                    high = cutoff;
                } else {
                    c = 2 * c + 2;
                    low = cutoff;
                }
            }
            if (t->node_count > t->nodes_before_lfill && !tree_is_leaf(t, c)) {
                double mL = quad_form(G + (2 * c + 1) * R2, xi, R);
                double cutoff = low + mL / m;
                if (d <= cutoff) {
                    c = 2 * c + 1;
                    high = cutoff;
                } else {
                    c = 2 * c + 2;
                    low = cutoff;
                }
            }
            int64_t leaf = tree_leaf_idx(t, c);
            int64_t res = 0;
            if (F > 1) {
                double frac = (d - low) / (high - low);
                int64_t rows = F < (t->n - leaf * F) ? F : (t->n - leaf * F);
                for (int64_t j = 0; j < F; j++) {
                    double v = 0.0;
                    if (j < rows) {
                        const double* u = U + (leaf * F + j) * R;
                        for (int64_t r = 0; r < R; r++) v += u[r] * xi[r];
                    }
                    q[j] = v;
                }
                double run = 0.0;
                for (int64_t j = 0; j < F; j++) {
                    double tmp = q[j] * q[j];
                    q[j] = run;
                    run += tmp;
                }
                for (int64_t j = 0; j < F; j++) q[j] /= run;
                res = F - 1;
                for (int64_t j = 0; j < F - 1; j++) {
                    if (frac < q[j + 1]) {
                        res = j;
                        break;
                    }
                }
            }
            int64_t row = res + leaf * F;
            out_idx[i] = (uint32_t)row;
            for (int64_t r = 0; r < R; r++) hmul[i * R + r] *= U[row * R + r];
        }
        free(q);
    }
}

/* ------------------------------------------------------------------------- */
/* Sorted lookup (sort_lookup.hpp:37-102): nonzeros ordered lexicographically */
/* by their coordinates with mode n left out.  Keys pack those coordinates,  */
/* most significant mode first, into 128 bits; an LSD radix sort keeps equal  */
/* keys in input order.                                                      */
/* ------------------------------------------------------------------------- */
static int bits_for(int64_t dim) {
    int b = 0;
    while (((int64_t)1 << b) < dim) b++;
    return b;
}

/* Packs the coordinates of mode != skip (skip = -1 packs all) of each row. */
int or_pack_keys(int N, int skip, const int64_t* dims, int64_t count, const uint32_t* idx, uint64_t* hi,
                 uint64_t* lo) {
    int total = 0;
    for (int k = 0; k < N; k++)
        if (k != skip) total += bits_for(dims[k]);
    if (total > 128) return -1;
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < count; i++) {
        uint64_t h = 0, l = 0;
        for (int k = 0; k < N; k++) {
            if (k == skip) continue;
            int b = bits_for(dims[k]);
            /* (h,l) <<= b, then | coord */
            if (b > 0) {
                if (b >= 64) {
                    h = l;
                    l = 0;
                } else {
                    h = (h << b) | (l >> (64 - b));
                    l <<= b;
                }
            }
            l |= (uint64_t)idx[i * N + k];
        }
        hi[i] = h;
        lo[i] = l;
    }
    return total;
}

/* Stable LSD radix sort of (hi, lo) keys over their low `bits` bits; returns
 * the permutation in perm (perm[i] = input position of the i-th smallest). */
void or_radix_sort128(int64_t count, int bits, const uint64_t* hi, const uint64_t* lo, int64_t* perm) {
    const int D = 11, B = 1 << D;
    int64_t* tmp = (int64_t*)malloc(sizeof(int64_t) * (size_t)(count > 0 ? count : 1));
    for (int64_t i = 0; i < count; i++) perm[i] = i;
    int nthreads = omp_get_max_threads();
    int64_t* hist = (int64_t*)malloc(sizeof(int64_t) * (size_t)nthreads * B);
    int64_t *src = perm, *dst = tmp;
    for (int shift = 0; shift < bits; shift += D) {
        memset(hist, 0, sizeof(int64_t) * (size_t)nthreads * B);
#pragma omp parallel num_threads(nthreads)
        {
            int tid = omp_get_thread_num();
            int64_t chunk = (count + nthreads - 1) / nthreads;
            int64_t s = chunk * tid < count ? chunk * tid : count;
            int64_t e = chunk * (tid + 1) < count ? chunk * (tid + 1) : count;
            int64_t* hh = hist + (int64_t)tid * B;
            for (int64_t i = s; i < e; i++) {
                int64_t p = src[i];
                uint64_t dg = shift >= 64 ? (hi[p] >> (shift - 64)) : (shift > 0 ? ((lo[p] >> shift) | (hi[p] << (64 - shift))) : lo[p]);
                hh[dg & (B - 1)]++;
            }
#pragma omp barrier
#pragma omp single
            {
                int64_t run = 0;
                for (int d = 0; d < B; d++)
                    for (int th = 0; th < nthreads; th++) {
                        int64_t c = hist[(int64_t)th * B + d];
                        hist[(int64_t)th * B + d] = run;
                        run += c;
                    }
            }
            for (int64_t i = s; i < e; i++) {
                int64_t p = src[i];
                uint64_t dg = shift >= 64 ? (hi[p] >> (shift - 64)) : (shift > 0 ? ((lo[p] >> shift) | (hi[p] << (64 - shift))) : lo[p]);
                dst[hh[dg & (B - 1)]++] = p;
            }
        }
        int64_t* sw = src;
        src = dst;
        dst = sw;
    }
    if (src != perm) memcpy(perm, src, sizeof(int64_t) * (size_t)count);
    free(hist);
    free(tmp);
}

/* Gathers rows/values by a permutation (the reorder=true branch,
 * sort_lookup.hpp:71-101). */
void or_apply_perm_u32(int64_t count, int width, const int64_t* perm, const uint32_t* in, uint32_t* out) {
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < count; i++) memcpy(out + i * width, in + perm[i] * width, sizeof(uint32_t) * width);
}
void or_apply_perm_f64(int64_t count, const int64_t* perm, const double* in, double* out) {
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < count; i++) out[i] = in[perm[i]];
}
void or_apply_perm_u64(int64_t count, const int64_t* perm, const uint64_t* in, uint64_t* out) {
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < count; i++) out[i] = in[perm[i]];
}

static inline int key_less(uint64_t ah, uint64_t al, uint64_t bh, uint64_t bl) {
    return ah < bh || (ah == bh && al < bl);
}

/* csr_based_spmm (sort_lookup.hpp:238-375).  For each (deduplicated) sample j
 * find every nonzero whose packed non-n key equals the sample's (equal_range
 * over the sorted keys), emit (row, j, value) triples, counting-sort them by
 * output row, then out[row] += value * design[j] with rows split across
 * threads.  Within a row, contributions are added in increasing j — the order
 * the reference produces.  `out` must be zeroed; returns the hit count. */
int64_t or_sampled_mttkrp(int64_t nnz, const uint64_t* khi, const uint64_t* klo, const uint32_t* rows_sorted,
                          const double* vals_sorted, int64_t Ju, const uint64_t* shi, const uint64_t* slo, int R,
                          const double* design, int64_t out_rows, double* out) {
    int64_t* start = (int64_t*)malloc(sizeof(int64_t) * (size_t)(Ju + 1));
    int64_t* cnt = (int64_t*)malloc(sizeof(int64_t) * (size_t)(Ju + 1));
#pragma omp parallel for schedule(static)
    for (int64_t j = 0; j < Ju; j++) {
        int64_t lo = 0, hi = nnz;
        while (lo < hi) { /* lower_bound */
            int64_t mid = lo + (hi - lo) / 2;
            if (key_less(khi[mid], klo[mid], shi[j], slo[j])) lo = mid + 1;
            else hi = mid;
        }
        int64_t s = lo;
        hi = nnz;
        while (lo < hi) { /* upper_bound */
            int64_t mid = lo + (hi - lo) / 2;
            if (key_less(shi[j], slo[j], khi[mid], klo[mid])) hi = mid;
            else lo = mid + 1;
        }
        start[j] = s;
        cnt[j] = lo - s;
    }
    int64_t H = 0;
    for (int64_t j = 0; j < Ju; j++) {
        int64_t c = cnt[j];
        cnt[j] = H;
        H += c;
    }
    cnt[Ju] = H;
    /* Triples in sample order. */
    uint32_t* trow = (uint32_t*)malloc(sizeof(uint32_t) * (size_t)(H > 0 ? H : 1));
    uint32_t* tcol = (uint32_t*)malloc(sizeof(uint32_t) * (size_t)(H > 0 ? H : 1));
    double* tval = (double*)malloc(sizeof(double) * (size_t)(H > 0 ? H : 1));
#pragma omp parallel for schedule(static)
    for (int64_t j = 0; j < Ju; j++) {
        int64_t o = cnt[j], len = cnt[j + 1] - cnt[j];
        for (int64_t p = 0; p < len; p++) {
            trow[o + p] = rows_sorted[start[j] + p];
            tcol[o + p] = (uint32_t)j;
            tval[o + p] = vals_sorted[start[j] + p];
        }
    }
    /* Counting sort by output row (parallel_sparse_transpose, sort_lookup.hpp:180-236). */
    int64_t* rowptr = (int64_t*)calloc((size_t)(out_rows + 1), sizeof(int64_t));
    for (int64_t h = 0; h < H; h++) rowptr[trow[h] + 1]++;
    for (int64_t r = 0; r < out_rows; r++) rowptr[r + 1] += rowptr[r];
    int64_t* fill = (int64_t*)malloc(sizeof(int64_t) * (size_t)(out_rows + 1));
    memcpy(fill, rowptr, sizeof(int64_t) * (size_t)(out_rows + 1));
    uint32_t* scol = (uint32_t*)malloc(sizeof(uint32_t) * (size_t)(H > 0 ? H : 1));
    double* sval = (double*)malloc(sizeof(double) * (size_t)(H > 0 ? H : 1));
    for (int64_t h = 0; h < H; h++) {
        int64_t pos = fill[trow[h]]++;
        scol[pos] = tcol[h];
        sval[pos] = tval[h];
    }
#pragma omp parallel for schedule(dynamic, 1024)
    for (int64_t r = 0; r < out_rows; r++) {
        double* o = out + r * R;
        for (int64_t p = rowptr[r]; p < rowptr[r + 1]; p++) {
            const double* d = design + (int64_t)scol[p] * R;
            double v = sval[p];
            for (int k = 0; k < R; k++) o[k] += d[k] * v;
        }
    }
    free(start);
    free(cnt);
    free(trow);
    free(tcol);
    free(tval);
    free(rowptr);
    free(fill);
    free(scol);
    free(sval);
    return H;
}

/* compute_2bmb (sort_lookup.hpp:377-438): sum over nonzeros of
 * x^2 - 2 x m(x), m(x) = sum_u sigma_u prod_k U_k[idx_k, u]; the partial
 * product over modes != 0 is formed first, then dotted with U_0's row. */
double or_fit_residual(int N, int R, int64_t nnz, const uint32_t* idx, const double* val, const double** U,
                       const double* sigma) {
    double total = 0.0;
#pragma omp parallel reduction(+ : total)
    {
        double* part = (double*)malloc(sizeof(double) * (size_t)R);
#pragma omp for schedule(static)
        for (int64_t i = 0; i < nnz; i++) {
            for (int u = 0; u < R; u++) part[u] = sigma[u];
            for (int k = 1; k < N; k++) {
                const double* row = U[k] + (int64_t)idx[i * N + k] * R;
                for (int u = 0; u < R; u++) part[u] *= row[u];
            }
            const double* row0 = U[0] + (int64_t)idx[i * N + 0] * R;
            double value = 0.0;
            for (int u = 0; u < R; u++) value += part[u] * row0[u];
            double x = val[i];
            total += x * x - 2 * value * x;
        }
        free(part);
    }
    return total;
}

/* execute_exact_mttkrp (sort_lookup.hpp:440-495): out[idx_n] += x * prod_{k!=n} U_k[idx_k]
 * over all nonzeros (rows of `out` are owned by threads through row hashing to
 * avoid atomics; the order within a row follows the nonzero order). */
void or_exact_mttkrp(int N, int mode, int R, int64_t nnz, const uint32_t* idx, const double* val, const double** U,
                     int64_t out_rows, double* out) {
    int nthreads = omp_get_max_threads();
#pragma omp parallel num_threads(nthreads)
    {
        int tid = omp_get_thread_num();
        double* part = (double*)malloc(sizeof(double) * (size_t)R);
        for (int64_t i = 0; i < nnz; i++) {
            int64_t r = idx[i * N + mode];
            if (r % nthreads != tid) continue;
            for (int u = 0; u < R; u++) part[u] = 1.0;
            for (int k = 0; k < N; k++) {
                if (k == mode) continue;
                const double* row = U[k] + (int64_t)idx[i * N + k] * R;
                for (int u = 0; u < R; u++) part[u] *= row[u];
            }
            double x = val[i];
            for (int u = 0; u < R; u++) out[r * R + u] += part[u] * x;
        }
        free(part);
    }
}

/* compute_DAGAT (common.h:727-746): res_i = a_i^T G a_i, G symmetric. */
void or_dagat(int64_t J, int R, const double* A, const double* G, double* res) {
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < J; i++) {
        const double* a = A + i * R;
        double acc = 0.0;
        for (int u = 0; u < R; u++) {
            double t = 0.0;
            for (int v = 0; v < R; v++) t += a[v] * G[u * R + v];
            acc += a[u] * t;
        }
        res[i] = acc;
    }
}

int or_num_threads(void) { return omp_get_max_threads(); }
