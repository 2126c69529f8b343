// ref_glue.cpp — C entry points over the reference sources compiled here
// (test infrastructure; built by ref_build.py into oracle/_ref/, never
// shipped).  The reference code itself is included from its own files:
//   sptrans.h            sptrans_scanTrans_specialized (the host transpose)
//   kernel.cu            the seven MLEM kernels, run on the CPU through
//                        ref_shim/cuda_runtime.h (one emulated thread at a time)
//   csr4matrix.cpp/.hpp  the csr4 reader
// The MLEM driver below restates the single-device loop of mlem()
// (main.cu:236-449, grids of main.cu:302-321) around the reference kernels.
#include <omp.h>

#include <cstdint>
#include <cstring>
#include <vector>

#include "cuda_runtime.h"
#include "kernel.cuh"
#include "sptrans.h"
#include "csr4matrix.hpp"

ref_emu_dim threadIdx, blockIdx, blockDim, gridDim;

// Runs kernel body k for every thread of the grid.  reverse = threads of a
// block in descending order, so lane 0 of each warp runs after lanes 1..31
// (mat_vec_mul_csr_vector reads the other lanes' partial sums).
template <class K>
static void launch(unsigned grid, unsigned block, bool reverse, K k) {
    gridDim = {grid, 1, 1};
    blockDim = {block, 1, 1};
    for (unsigned b = 0; b < grid; ++b) {
        blockIdx = {b, 0, 0};
        for (unsigned q = 0; q < block; ++q) {
            threadIdx = {reverse ? block - 1 - q : q, 0, 0};
            k();
        }
    }
}

static unsigned cdiv(uint64_t a, uint64_t b) { return (unsigned)((a + b - 1) / b); }

extern "C" {

void ref_sptrans(int nthreads, uint32_t m, uint32_t n, uint64_t nnz, const uint64_t* rowptr,
                 const uint32_t* col, const float* val, uint32_t* rowT, uint64_t* colptr, float* valT) {
    omp_set_num_threads(nthreads);
    std::memset(colptr, 0, sizeof(uint64_t) * ((size_t)n + 1));  // main.cu:101 calloc
    sptrans_scanTrans_specialized(m, n, nnz, (unsigned long*)rowptr, (unsigned int*)col, (float*)val,
                                  rowT, (unsigned long*)colptr, valT);
}

int ref_csr4_header(const char* path, uint32_t* rows, uint32_t* cols, uint64_t* nnz) {
    try {
        Csr4Matrix m(path);
        *rows = m.rows();
        *cols = m.columns();
        *nnz = m.elements();
        return 0;
    } catch (...) {
        return 1;
    }
}

// csr_format_for_cuda (main.cu:518-554) over the reference reader.
int ref_csr4_read(const char* path, uint64_t* rowptr, uint32_t* col, float* val) {
    try {
        Csr4Matrix m(path);
        m.mapRows(0, m.rows());
        rowptr[0] = 0;
        for (uint32_t r = 0; r < m.rows(); ++r) rowptr[r + 1] = rowptr[r] + m.elementsInRow(r);
        for (uint32_t r = 0; r < m.rows(); ++r) {
            uint64_t k = rowptr[r];
            for (auto it = m.beginRow2(r); it != m.endRow2(r); ++it, ++k) {
                col[k] = (uint32_t)(*it).column();
                val[k] = (*it).value();
            }
        }
        return 0;
    } catch (...) {
        return 1;
    }
}

// y = A x through a reference kernel: spmv 0 merge-based (grid of
// main.cu:306), 1 csr-vector (main.cu:308); scatter = 1 runs
// calcBwProj_none_trans instead (y += Aᵀ x, main.cu:320).
void ref_spmv(int spmv, int scatter, uint32_t secsize, const uint64_t* rowptr64, const uint32_t* col,
              const float* val, const float* x, uint32_t rows, uint64_t nnz, float* y) {
    std::vector<unsigned> rp(rows + 1);
    for (uint32_t r = 0; r <= rows; ++r) rp[r] = (unsigned)rowptr64[r];
    unsigned* C = const_cast<unsigned*>(col);
    float* V = const_cast<float*>(val);
    float* X = const_cast<float*>(x);
    if (scatter) {
        launch(cdiv(rows, 32), 1024, false, [&] { calcBwProj_none_trans(rp.data(), C, V, X, y, rows); });
    } else if (spmv == 0) {
        launch(cdiv(rows + nnz, 1024ull * secsize), 1024, false,
               [&] { calcFwProj_merge_based(rp.data(), C, V, X, y, secsize, rows, (unsigned)nnz); });
    } else {
        launch(cdiv(rows, 32), 1024, true, [&] { calcFwProj_csr_vector(rp.data(), C, V, X, y, rows); });
    }
}

// Single-device mlem() loop (main.cu:329-449) over the reference kernels.
void ref_mlem(const uint64_t* rowptr64, const uint32_t* col, const float* val, const uint64_t* rowptrT64,
              const uint32_t* colT, const float* valT, const int32_t* g, const float* norm, float* f,
              uint32_t rows, uint32_t cols, uint64_t nnz, uint32_t iterations, uint32_t matrix_vector_mul,
              uint32_t secsize_fp, uint32_t secsize_bp, uint32_t using_trans) {
    const unsigned bs = 1024;
    std::vector<unsigned> rp(rows + 1), rpT(using_trans == 0 ? cols + 1 : 1);
    for (uint32_t r = 0; r <= rows; ++r) rp[r] = (unsigned)rowptr64[r];
    if (using_trans == 0)
        for (uint32_t c = 0; c <= cols; ++c) rpT[c] = (unsigned)rowptrT64[c];
    unsigned* C = const_cast<unsigned*>(col);
    float* V = const_cast<float*>(val);
    unsigned* CT = const_cast<unsigned*>(colT);
    float* VT = const_cast<float*>(valT);
    std::vector<int> gv(g, g + rows);
    std::vector<float> fv(f, f + cols), nm(norm, norm + cols), temp(rows, 0.0f), bw(cols, 0.0f);
    const unsigned g_correl = cdiv(rows, bs);
    const unsigned g_fp = matrix_vector_mul == 0 ? cdiv(rows + nnz, (uint64_t)bs * secsize_fp) : cdiv(rows, 32);
    const unsigned g_update = cdiv(cols, bs);
    const unsigned g_bp = using_trans == 0
                              ? (matrix_vector_mul == 0 ? cdiv(cols + nnz, (uint64_t)bs * secsize_bp) : cdiv(cols, 32))
                              : cdiv(rows, 32);
    for (uint32_t it = 0; it < iterations; ++it) {
        if (matrix_vector_mul == 0)
            launch(g_fp, bs, false, [&] {
                calcFwProj_merge_based(rp.data(), C, V, fv.data(), temp.data(), secsize_fp, rows, (unsigned)nnz);
            });
        else
            launch(g_fp, bs, true, [&] { calcFwProj_csr_vector(rp.data(), C, V, fv.data(), temp.data(), rows); });
        launch(g_correl, bs, false, [&] { calcCorrel(gv.data(), temp.data(), rows); });
        if (using_trans == 0) {
            if (matrix_vector_mul == 0)
                launch(g_bp, bs, false, [&] {
                    calcBwProj_merge_based(rpT.data(), CT, VT, temp.data(), bw.data(), secsize_bp, cols, (unsigned)nnz);
                });
            else
                launch(g_bp, bs, true, [&] { calcBwProj_csr_vector(rpT.data(), CT, VT, temp.data(), bw.data(), cols); });
        } else {
            launch(g_bp, bs, false, [&] { calcBwProj_none_trans(rp.data(), C, V, temp.data(), bw.data(), rows); });
        }
        launch(g_update, bs, false, [&] { calcUpdate(fv.data(), nm.data(), bw.data(), cols); });
        fv = bw;  // single-rank ncclAllReduce(bwproj -> f), main.cu:426-429
        std::fill(bw.begin(), bw.end(), 0.0f);
        std::fill(temp.begin(), temp.end(), 0.0f);
    }
    std::memcpy(f, fv.data(), sizeof(float) * cols);
}

}  // extern "C"
