// cli_main.cpp — command-line drop-in for the reference binary ./test.
//
// Same eight positional arguments and checks as main() (main.cu:42-62), the
// same help text on bad input (help(), main.cu:614-625) and the same result
// line "\nSum f: %f\n" (main.cu:460-463).  The matrix is read from the csr4
// file, uploaded once, transposed and normalised on the GPU; the initial image
// is the reference's Σg/Σnorm (main.cu:83-97).  When the file's scanner
// configuration gives a voxel grid with nx*ny*nz = columns, the matrix goes
// into the locality layout (voxel bricks, LORs ordered by where they cross the
// grid); the result differs from the natural layout only by FP32 rounding.
// Setting MLEM_WRITE_IMAGE=path also writes the image as raw float32
// (vector.hpp:77-87 format).
#include <cstdio>
#include <cstdlib>
#include <string>
#include <vector>

#include "../../include/mlem.h"

static void help() {
    std::printf("\nWrong parameters! Please read the following instructions:\n\n");
    std::printf("total amount of parameters: 9\n");
    std::printf("argv[1]: path of matrix file\n");
    std::printf("argv[2]: path of image  file\n");
    std::printf("argv[3]: iteration times\n");
    std::printf("argv[4]: number of GPUs to be used\n");
    std::printf("argv[5]: section size for forward  projection (merge-based SpMV)\n");
    std::printf("argv[6]: section size for backward projection (merge-based SpMV)\n");
    std::printf("argv[7]: BP uses transposed matrix?      0: yes                1: no\n");
    std::printf("argv[8]: which SpMV algorithm to use?    0: merge-based SpMV   1: csr-vector SpMV\n\n");
}

static int die(const char* what, mlem_status st) {
    std::fprintf(stderr, "%s failed (%d): %s\n", what, (int)st, mlem_last_error());
    return EXIT_FAILURE;
}

int main(int argc, char** argv) {
    if (argc != 9) {
        help();
        return EXIT_FAILURE;
    }
    const unsigned iterations = (unsigned)std::strtol(argv[3], nullptr, 10);
    const unsigned devices = (unsigned)std::strtol(argv[4], nullptr, 10);
    const unsigned secsize_fp = (unsigned)std::strtol(argv[5], nullptr, 10);
    const unsigned secsize_bp = (unsigned)std::strtol(argv[6], nullptr, 10);
    const unsigned using_trans = (unsigned)std::strtol(argv[7], nullptr, 10);
    const unsigned spmv = (unsigned)std::strtol(argv[8], nullptr, 10);
    if (iterations == 0 || devices == 0 || secsize_fp == 0 || secsize_bp == 0 ||
        (using_trans != 0 && using_trans != 1) || (spmv != 0 && spmv != 1)) {
        help();
        return EXIT_FAILURE;
    }
    if (devices != 1) {
        // one process drives one GPU; larger jobs run as independent replicas
        help();
        return EXIT_FAILURE;
    }
    mlem_matrix_opts mo;
    mlem_matrix_opts_default(&mo);
    mo.build_transpose = using_trans == 0 ? 1 : 0;
    mlem_csr4_header hdr;
    mlem_status st = mlem_csr4_read_header(argv[1], &hdr);
    if (st != MLEM_OK) return die("loading the matrix", st);
    if (hdr.nx && hdr.ny && hdr.nz && (uint64_t)hdr.nx * hdr.ny * hdr.nz == hdr.cols) mo.layout = MLEM_LAYOUT_LOCALITY;
    mlem_matrix* m = nullptr;
    st = mlem_matrix_load_csr4(argv[1], &mo, &m);
    if (st != MLEM_OK) return die("loading the matrix", st);
    mlem_matrix_info info;
    mlem_matrix_get_info(m, &info);
    uint64_t n = 0;
    st = mlem_read_sinogram(argv[2], nullptr, 0, &n);
    if (st != MLEM_OK) return die("reading the image file", st);
    if (n < info.rows) {
        std::fprintf(stderr, "image file holds %llu values, the matrix has %u rows\n",
                     (unsigned long long)n, info.rows);
        mlem_matrix_destroy(m);
        return EXIT_FAILURE;
    }
    std::vector<int32_t> g(n);
    st = mlem_read_sinogram(argv[2], g.data(), n, &n);
    if (st != MLEM_OK) return die("reading the image file", st);
    mlem_run_opts ro;
    mlem_run_opts_default(&ro);
    ro.spmv = spmv ? MLEM_SPMV_CSR_VECTOR : MLEM_SPMV_MERGE;
    ro.bp_mode = using_trans ? MLEM_BP_SCATTER : MLEM_BP_TRANS;
    ro.secsize_fp = secsize_fp;
    ro.secsize_bp = secsize_bp;
    std::vector<float> f(info.cols);
    st = mlem_run(m, g.data(), nullptr, iterations, &ro, f.data(), nullptr, nullptr);
    if (st != MLEM_OK) return die("mlem_run", st);
    float sum = 0.0f;
    for (unsigned i = 0; i < info.cols; ++i) sum += f[i];
    std::printf("\nSum f: %f\n", sum);
    if (const char* out = std::getenv("MLEM_WRITE_IMAGE")) {
        st = mlem_write_image(out, f.data(), f.size());
        if (st != MLEM_OK) return die("writing the image", st);
    }
    mlem_matrix_destroy(m);
    return EXIT_SUCCESS;
}
