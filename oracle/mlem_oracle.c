/*
 * mlem_oracle.c — CPU restatement of the reference MLEM path.
 *
 * TEST INFRASTRUCTURE ONLY.  Nothing in the product library calls this code;
 * it is the checker that tests/, __graft_entry__.smoke() and the CPU legs of
 * bench.py compare the CUDA path against.  Each function cites the reference
 * file:line it restates (wmd0701/Bachelorarbeit-MLEM).  It is pinned against
 * the reference itself: sptrans.h and kernel.cu compiled here from their own
 * sources (oracle/ref_build.py) produced the committed fixtures in
 * tests/golden/, and tests check this file against them bit for bit.
 *
 * Floating point: compiled with -ffp-contract=off.  Functions that restate a
 * CUDA kernel take use_fma: 1 reproduces nvcc's default contraction of
 * `acc += a*b` into fmaf(a, b, acc); 0 keeps a separate multiply and add
 * (the order the reference kernels have when compiled for the host).
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

int oracle_max_threads(void);

static inline float madd(float acc, float a, float b, int use_fma) {
    return use_fma ? fmaf(a, b, acc) : acc + a * b;
}

/* ------------------------------------------------------------ transpose */
/* Stable counting sort of the nonzeros by column: the permutation produced by
 * sptrans_scanTrans_specialized (sptrans.h:397-545) — per-thread column
 * histograms over contiguous row ranges (sptrans.h:432-449), their prefix
 * over columns and threads (sptrans.h:450-463), and the write-back of each
 * thread's rows in original order (sptrans.h:465-545).  Entries of a column
 * keep their original order, so the output does not depend on the thread
 * count. */
void oracle_transpose(uint32_t rows, uint32_t cols, uint64_t nnz, const uint64_t* rowptr,
                      const uint32_t* col, const float* val, uint64_t* colptr, uint32_t* rowT,
                      float* valT) {
    int T = omp_get_max_threads();
    if (T < 1) T = 1;
    if ((uint64_t)T > (uint64_t)rows) T = rows ? (int)rows : 1;
    /* nnz-balanced contiguous row ranges */
    uint32_t* rb = (uint32_t*)malloc(sizeof(uint32_t) * ((size_t)T + 1));
    rb[0] = 0;
    for (int t = 1; t < T; ++t) {
        const uint64_t target = nnz * (uint64_t)t / (uint64_t)T;
        uint32_t lo = rb[t - 1], hi = rows;
        while (lo < hi) {
            const uint32_t mid = lo + (hi - lo) / 2;
            if (rowptr[mid] < target) lo = mid + 1;
            else hi = mid;
        }
        rb[t] = lo;
    }
    rb[T] = rows;
    uint64_t* cnt = (uint64_t*)calloc((size_t)T * ((size_t)cols + 1), sizeof(uint64_t));
#pragma omp parallel for num_threads(T) schedule(static, 1)
    for (int t = 0; t < T; ++t) {
        uint64_t* h = cnt + (size_t)t * ((size_t)cols + 1);
        for (uint64_t e = rowptr[rb[t]]; e < rowptr[rb[t + 1]]; ++e) h[col[e]]++;
    }
    /* column-major prefix: column c of thread t starts after all of columns
     * < c and after column c of threads < t */
    uint64_t run = 0;
    for (uint32_t c = 0; c < cols; ++c) {
        colptr[c] = run;
        for (int t = 0; t < T; ++t) {
            uint64_t* h = cnt + (size_t)t * ((size_t)cols + 1);
            const uint64_t k = h[c];
            h[c] = run;
            run += k;
        }
    }
    colptr[cols] = run;
#pragma omp parallel for num_threads(T) schedule(static, 1)
    for (int t = 0; t < T; ++t) {
        uint64_t* cur = cnt + (size_t)t * ((size_t)cols + 1);
        for (uint32_t r = rb[t]; r < rb[t + 1]; ++r)
            for (uint64_t e = rowptr[r]; e < rowptr[r + 1]; ++e) {
                const uint64_t p = cur[col[e]]++;
                rowT[p] = r;
                if (val) valT[p] = val[e];
            }
    }
    free(cnt);
    free(rb);
}

/* ---------------------------------------------------------- merge search */
/* merge_based_start search loop (kernel.cu:202-229) for thread starts
 * t*secsize.  The reference may read csr_Rows[rows+1]; that probe only occurs
 * when i == rows and every outcome ends the loop there, so it is answered
 * without the read. */
static void search_one(const uint64_t* rowptr, uint32_t rows, int64_t start, int64_t* oi, int64_t* oj) {
    int64_t lefti = 0, righti = rows, nexti = righti / 2, nextj = start - nexti, i = 0, j = start;
    while (i != nexti) {
        i = nexti;
        j = nextj;
        const int right = (i + 1 > (int64_t)rows) ? 1 : ((int64_t)rowptr[i + 1] > j - 1);
        if (right) righti = i;
        else lefti = i + 1;
        nexti = (lefti + righti) / 2;
        nextj = start - nexti;
    }
    *oi = i;
    *oj = j;
}

void oracle_merge_search(const uint64_t* rowptr, uint32_t rows, uint32_t secsize, uint64_t nthreads,
                         int64_t* oi, int64_t* oj) {
    for (uint64_t t = 0; t < nthreads; ++t) search_one(rowptr, rows, (int64_t)(t * secsize), oi + t, oj + t);
}

/* Merrill & Garland MergePathSearch (2016), used only to cross-check the
 * restatement above: A = row end offsets, B = nonzero indices. */
void oracle_merge_search_mg(const uint64_t* rowptr, uint32_t rows, uint64_t nnz, uint32_t secsize,
                            uint64_t nthreads, int64_t* oi, int64_t* oj) {
    for (uint64_t t = 0; t < nthreads; ++t) {
        const int64_t d = (int64_t)(t * secsize);
        int64_t lo = d - (int64_t)nnz > 0 ? d - (int64_t)nnz : 0;
        int64_t hi = d < (int64_t)rows ? d : (int64_t)rows;
        while (lo < hi) {
            const int64_t piv = (lo + hi) / 2;
            if ((int64_t)rowptr[piv + 1] <= d - piv - 1) lo = piv + 1;
            else hi = piv;
        }
        oi[t] = lo;
        oj[t] = d - lo;
    }
}

/* ------------------------------------------------------------- products */
/* mat_vec_mul_csr_vector (kernel.cu:297-336): lane l of the row's warp sums
 * elements start+l, start+l+32, ...; lane 0 then adds lanes 1..31 in order. */
void oracle_spmv_csrvec(const uint64_t* rowptr, const uint32_t* col, const float* val, const float* x,
                        uint32_t rows, float* y, int use_fma) {
#pragma omp parallel for schedule(static)
    for (int64_t r = 0; r < (int64_t)rows; ++r) {
        float lane[32];
        for (int l = 0; l < 32; ++l) {
            float acc = 0.0f;
            for (uint64_t e = rowptr[r] + l; e < rowptr[r + 1]; e += 32)
                acc = madd(acc, val[e], x[col[e]], use_fma);
            lane[l] = acc;
        }
        float s = lane[0];
        for (int l = 1; l < 32; ++l) s += lane[l];
        y[r] = 0.0f + s; /* atomicAdd into a zeroed output */
    }
}

/* merge_based_work (kernel.cu:257-286) of every thread, its atomicAdd's
 * applied in ascending thread order; y must be zeroed by the caller
 * (main.cu:291-297, 436-448). */
void oracle_spmv_merge(const uint64_t* rowptr, const uint32_t* col, const float* val, const float* x,
                       uint32_t rows, uint64_t nnz, uint32_t secsize, uint64_t nthreads, float* y,
                       int use_fma) {
    int64_t i, j;
    for (uint64_t t = 0; t < nthreads; ++t) {
        search_one(rowptr, rows, (int64_t)(t * secsize), &i, &j);
        uint64_t end = (uint64_t)(i + j) + secsize;
        if (end > nnz + rows) end = nnz + rows;
        float acc = 0.0f;
        while ((uint64_t)(i + j) < end) {
            if (rowptr[i + 1] > (uint64_t)j) {
                acc = madd(acc, val[j], x[col[j]], use_fma);
                j++;
            } else {
                y[i] += acc;
                i++;
                acc = 0.0f;
            }
        }
        if (acc != 0.0f) y[i] += acc;
    }
}

/* trans_mat_vec_mul_warp (kernel.cu:347-370): y[col] += val * x[row], rows in
 * order, lanes 0..31 in order, each lane's elements in order. */
void oracle_scatter(const uint64_t* rowptr, const uint32_t* col, const float* val, const float* x,
                    uint32_t rows, float* y) {
    for (uint32_t r = 0; r < rows; ++r)
        for (int l = 0; l < 32; ++l)
            for (uint64_t e = rowptr[r] + l; e < rowptr[r + 1]; e += 32) y[col[e]] += val[e] * x[r];
}

/* calcCorrel (kernel.cu:11-19). */
void oracle_correl(const int32_t* g, float* fp, uint32_t rows) {
    for (uint32_t i = 0; i < rows; ++i)
        if (fp[i] != 0.0f) fp[i] = (float)g[i] / fp[i];
}

/* calcUpdate (kernel.cu:28-39): result written to bp. */
void oracle_update(const float* f, const float* norm, float* bp, uint32_t cols) {
    for (uint32_t c = 0; c < cols; ++c) {
        if (norm[c] == 0.0f) bp[c] = f[c] * bp[c];
        else bp[c] = f[c] * bp[c] / norm[c];
    }
}

/* Sensitivity image Aᵀ1: calcColumnSums (main.cu:558-580) in FP32 with rows
 * in order (the reference's OpenMP reduction order is unspecified). */
void oracle_colsum_f32(const uint64_t* rowptr, const uint32_t* col, const float* val, uint32_t rows,
                       uint32_t cols, float* norm) {
    memset(norm, 0, sizeof(float) * cols);
    for (uint32_t r = 0; r < rows; ++r)
        for (uint64_t e = rowptr[r]; e < rowptr[r + 1]; ++e) norm[col[e]] += val[e];
}

/* Same sums accumulated in FP64, rounded once to FP32. */
void oracle_colsum_f64(const uint64_t* rowptr, const uint32_t* col, const float* val, uint32_t rows,
                       uint32_t cols, float* norm) {
    double* acc = (double*)calloc(cols ? cols : 1, sizeof(double));
    for (uint32_t r = 0; r < rows; ++r)
        for (uint64_t e = rowptr[r]; e < rowptr[r + 1]; ++e) acc[col[e]] += (double)val[e];
    for (uint32_t c = 0; c < cols; ++c) norm[c] = (float)acc[c];
    free(acc);
}

/* The same FP64 column sums from the rows of Aᵀ (OpenMP over columns).  A
 * stable transpose lists each column's entries in increasing row order, the
 * order oracle_colsum_f64 adds them in, so both give the same bits. */
void oracle_colsum_f64_t(const uint64_t* rowptrT, const float* valT, uint32_t cols, float* norm) {
#pragma omp parallel for schedule(dynamic, 4096)
    for (int64_t c = 0; c < (int64_t)cols; ++c) {
        double s = 0.0;
        for (uint64_t e = rowptrT[c]; e < rowptrT[c + 1]; ++e) s += (double)valT[e];
        norm[c] = (float)s;
    }
}

/* Initial image value (main.cu:83-97): FP32 running sum of norm, int sum of
 * g, init = sum_g / sum_norm. */
float oracle_initial_value(const int32_t* g, uint32_t rows, const float* norm, uint32_t cols) {
    float sum_norm = 0.0f;
    int64_t sum_g = 0;
    for (uint32_t c = 0; c < cols; ++c) sum_norm += norm[c];
    for (uint32_t r = 0; r < rows; ++r) sum_g += g[r];
    return (float)sum_g / sum_norm;
}

/* ---------------------------------------------------------------- MLEM */
/* The single-device iteration loop of mlem() (main.cu:329-449) in FP32 with
 * the kernels restated above.  Grid sizes follow main.cu:302-321 (blocksize
 * 1024).  f holds f0 on entry and the image on exit. */
void oracle_mlem_f32(const uint64_t* rowptr, const uint32_t* col, const float* val,
                     const uint64_t* rowptrT, const uint32_t* colT, const float* valT,
                     const int32_t* g, const float* norm, float* f, uint32_t rows, uint32_t cols,
                     uint64_t nnz, uint32_t iterations, uint32_t matrix_vector_mul,
                     uint32_t secsize_fp, uint32_t secsize_bp, uint32_t using_trans, int use_fma) {
    float* temp = (float*)calloc(rows ? rows : 1, sizeof(float));
    float* bp = (float*)calloc(cols ? cols : 1, sizeof(float));
    const uint64_t fp_threads = ((rows + nnz + 1024ull * secsize_fp - 1) / (1024ull * secsize_fp)) * 1024ull;
    const uint64_t bp_threads = ((cols + nnz + 1024ull * secsize_bp - 1) / (1024ull * secsize_bp)) * 1024ull;
    for (uint32_t it = 0; it < iterations; ++it) {
        if (matrix_vector_mul == 0)
            oracle_spmv_merge(rowptr, col, val, f, rows, nnz, secsize_fp, fp_threads, temp, use_fma);
        else
            oracle_spmv_csrvec(rowptr, col, val, f, rows, temp, use_fma);
        oracle_correl(g, temp, rows);
        if (using_trans == 0) {
            if (matrix_vector_mul == 0)
                oracle_spmv_merge(rowptrT, colT, valT, temp, cols, nnz, secsize_bp, bp_threads, bp, use_fma);
            else
                oracle_spmv_csrvec(rowptrT, colT, valT, temp, cols, bp, use_fma);
        } else {
            oracle_scatter(rowptr, col, val, temp, rows, bp);
        }
        oracle_update(f, norm, bp, cols);
        memcpy(f, bp, sizeof(float) * cols); /* single-rank AllReduce bp -> f */
        memset(bp, 0, sizeof(float) * cols);
        memset(temp, 0, sizeof(float) * rows);
    }
    free(temp);
    free(bp);
}

/* FP64 oracle of record: the same MLEM update with every quantity in double
 * (forward projection, ratio, back projection, update), back projection by
 * rows of A (exact in any order up to double rounding).  f0 and f_out are
 * double; norm is taken in double.  loglik (optional, [iterations]) receives
 * Σ g log(Af) - Af of the image entering each iteration (rows with Af > 0). */
void oracle_mlem_f64(const uint64_t* rowptr, const uint32_t* col, const float* val, const int32_t* g,
                     const double* norm, const double* f0, uint32_t rows, uint32_t cols,
                     uint32_t iterations, double* f_out, double* loglik) {
    double* f = (double*)malloc(sizeof(double) * (cols ? cols : 1));
    double* ratio = (double*)malloc(sizeof(double) * (rows ? rows : 1));
    double* bp = (double*)malloc(sizeof(double) * (cols ? cols : 1));
    memcpy(f, f0, sizeof(double) * cols);
    for (uint32_t it = 0; it < iterations; ++it) {
        double ll = 0.0;
#pragma omp parallel for schedule(static) reduction(+ : ll)
        for (int64_t r = 0; r < (int64_t)rows; ++r) {
            double s = 0.0;
            for (uint64_t e = rowptr[r]; e < rowptr[r + 1]; ++e) s += (double)val[e] * f[col[e]];
            ratio[r] = s != 0.0 ? (double)g[r] / s : 0.0;
            if (s > 0.0) ll += (g[r] > 0 ? (double)g[r] * log(s) : 0.0) - s;
        }
        if (loglik) loglik[it] = ll;
        memset(bp, 0, sizeof(double) * cols);
        for (uint32_t r = 0; r < rows; ++r) {
            const double q = ratio[r];
            if (q == 0.0) continue;
            for (uint64_t e = rowptr[r]; e < rowptr[r + 1]; ++e) bp[col[e]] += (double)val[e] * q;
        }
        for (uint32_t c = 0; c < cols; ++c) f[c] = norm[c] == 0.0 ? f[c] * bp[c] : f[c] * bp[c] / norm[c];
    }
    memcpy(f_out, f, sizeof(double) * cols);
    free(f);
    free(ratio);
    free(bp);
}

/* The FP64 oracle with the back projection over rows of Aᵀ (parallel over
 * columns): the same quantities as oracle_mlem_f64, summed in another order,
 * so results agree to FP64 rounding.  For full-size matrices. */
void oracle_mlem_f64_t(const uint64_t* rowptr, const uint32_t* col, const float* val,
                       const uint64_t* rowptrT, const uint32_t* colT, const float* valT, const int32_t* g,
                       const double* norm, const double* f0, uint32_t rows, uint32_t cols,
                       uint32_t iterations, double* f_out, double* loglik) {
    double* f = (double*)malloc(sizeof(double) * (cols ? cols : 1));
    double* ratio = (double*)malloc(sizeof(double) * (rows ? rows : 1));
    memcpy(f, f0, sizeof(double) * cols);
    for (uint32_t it = 0; it < iterations; ++it) {
        double ll = 0.0;
#pragma omp parallel for schedule(dynamic, 1024) reduction(+ : ll)
        for (int64_t r = 0; r < (int64_t)rows; ++r) {
            double s = 0.0;
            for (uint64_t e = rowptr[r]; e < rowptr[r + 1]; ++e) s += (double)val[e] * f[col[e]];
            ratio[r] = s != 0.0 ? (double)g[r] / s : 0.0;
            if (s > 0.0) ll += (g[r] > 0 ? (double)g[r] * log(s) : 0.0) - s;
        }
        if (loglik) loglik[it] = ll;
#pragma omp parallel for schedule(dynamic, 1024)
        for (int64_t c = 0; c < (int64_t)cols; ++c) {
            double s = 0.0;
            for (uint64_t e = rowptrT[c]; e < rowptrT[c + 1]; ++e) s += (double)valT[e] * ratio[colT[e]];
            f[c] = norm[c] == 0.0 ? f[c] * s : f[c] * s / norm[c];
        }
    }
    memcpy(f_out, f, sizeof(double) * cols);
    free(f);
    free(ratio);
}

/* CPU baseline: transposed-form MLEM with FP32 values and image, FP64
 * accumulation, OpenMP over rows of A (forward) and rows of Aᵀ (back).
 * nthreads <= 0 uses the OpenMP default. */
void oracle_mlem_omp(const uint64_t* rowptr, const uint32_t* col, const float* val,
                     const uint64_t* rowptrT, const uint32_t* colT, const float* valT,
                     const int32_t* g, const float* norm, float* f, uint32_t rows, uint32_t cols,
                     uint32_t iterations, int nthreads) {
    /* the thread count applies to this call only (num_threads clauses), so a
     * one-thread run leaves the process default untouched */
    const int T = nthreads > 0 ? nthreads : oracle_max_threads();
    float* ratio = (float*)malloc(sizeof(float) * (rows ? rows : 1));
    for (uint32_t it = 0; it < iterations; ++it) {
#pragma omp parallel for num_threads(T) schedule(dynamic, 1024)
        for (int64_t r = 0; r < (int64_t)rows; ++r) {
            double s = 0.0;
            for (uint64_t e = rowptr[r]; e < rowptr[r + 1]; ++e) s += (double)val[e] * (double)f[col[e]];
            ratio[r] = s != 0.0 ? (float)((double)g[r] / s) : 0.0f;
        }
#pragma omp parallel for num_threads(T) schedule(dynamic, 1024)
        for (int64_t c = 0; c < (int64_t)cols; ++c) {
            double s = 0.0;
            for (uint64_t e = rowptrT[c]; e < rowptrT[c + 1]; ++e) s += (double)valT[e] * (double)ratio[colT[e]];
            const double t = (double)f[c] * s;
            f[c] = (float)(norm[c] == 0.0f ? t : t / (double)norm[c]);
        }
    }
    free(ratio);
}

int oracle_max_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

/* y = A·x in FP64 (OpenMP over rows): the expected counts of a phantom. */
void oracle_project_f64(const uint64_t* rowptr, const uint32_t* col, const float* val, const float* x,
                        uint32_t rows, double* y) {
#pragma omp parallel for schedule(dynamic, 1024)
    for (int64_t r = 0; r < (int64_t)rows; ++r) {
        double s = 0.0;
        for (uint64_t e = rowptr[r]; e < rowptr[r + 1]; ++e) s += (double)val[e] * (double)x[col[e]];
        y[r] = s;
    }
}
