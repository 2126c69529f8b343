// io.cu — on-disk formats and host-side helpers of the C ABI.
//
// csr4 (helper_files_common/csr4matrix.cpp:36-178, matrixelement.hpp:37-46),
// little-endian:
//   0  "PCSR"  4 version (=4)  5 symmetry flags  6-7 padding
//   8  u32 rows  12 u32 columns  16 u64 nnz  24 u32 scanner-config bytes
//   28 scanner config: u32 nLayers, {f32 w,h,d,r,mu} x nLayers, u32 nBlocks,
//      u32 blocksize, f32 x (blocksize-1) gaps, u32 nRings, f32 x (nRings-1)
//      gaps, f32 voxel w,h,d, u32 nx,ny,nz   (size must match exactly)
//   then u64 row END offsets [rows] (no leading 0), then nnz x {u32 col, f32 val}.
// The reader checks sizes in 64-bit arithmetic (the reference computes the
// expected file size in uint32_t, csr4matrix.cpp:95-96) and rejects
// non-monotone row offsets and column indices >= columns.
//
// Raw vectors (helper_files_common/vector.hpp:33-87): headerless arrays; a
// size that is not a multiple of the element size is an error.
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "runtime.h"

namespace mlem {
namespace {

struct File {
    FILE* f = nullptr;
    explicit File(const char* path, const char* mode) { f = std::fopen(path, mode); }
    ~File() {
        if (f) std::fclose(f);
    }
};

uint64_t file_size(FILE* f) {
    std::fseek(f, 0, SEEK_END);
    const long long n = ftello(f);
    std::fseek(f, 0, SEEK_SET);
    return n < 0 ? 0 : (uint64_t)n;
}

void read_exact(FILE* f, void* dst, uint64_t bytes, const std::string& what) {
    if (bytes && std::fread(dst, 1, bytes, f) != bytes) fail(MLEM_EIO, "short read: " + what);
}

template <typename T>
T rd(const std::vector<unsigned char>& b, uint64_t& p, const std::string& path) {
    if (p + sizeof(T) > b.size()) fail(MLEM_EIO, "Error reading scanner geometry configuration: " + path);
    T v;
    std::memcpy(&v, b.data() + p, sizeof(T));
    p += sizeof(T);
    return v;
}

struct Csr4Info {
    mlem_csr4_header h{};
    uint32_t scan_bytes = 0;
    uint64_t data_off = 0;
};

Csr4Info parse_header(const char* path) {
    File fh(path, "rb");
    if (!fh.f) fail(MLEM_EIO, std::string("Cannot open file ") + path);
    const uint64_t size = file_size(fh.f);
    if (size < 28) fail(MLEM_EIO, std::string("File too short ") + path);
    unsigned char hdr[28];
    read_exact(fh.f, hdr, 28, path);
    if (std::memcmp(hdr, "PCSR", 4) != 0)
        fail(MLEM_EIO, std::string("Input file '") + path + "' is not a CSR matrix");
    if (hdr[4] != 4) fail(MLEM_EIO, std::string("Input file '") + path + "' has wrong CSR version (need v4)");
    Csr4Info info;
    info.h.sym_flags = hdr[5];
    std::memcpy(&info.h.rows, hdr + 8, 4);
    std::memcpy(&info.h.cols, hdr + 12, 4);
    std::memcpy(&info.h.nnz, hdr + 16, 8);
    std::memcpy(&info.scan_bytes, hdr + 24, 4);
    if (info.scan_bytes < 60) fail(MLEM_EIO, "Cannot find scanner geometry configuration");
    const unsigned __int128 need = (unsigned __int128)28 + info.scan_bytes + (unsigned __int128)info.h.rows * 8 +
                                   (unsigned __int128)info.h.nnz * 8;
    if ((unsigned __int128)size < need)
        fail(MLEM_EIO, std::string("Input file '") + path + "' is too short");
    std::vector<unsigned char> sc(info.scan_bytes);
    read_exact(fh.f, sc.data(), sc.size(), path);
    uint64_t p = 0;
    const std::string ps(path);
    const uint32_t nlayers = rd<uint32_t>(sc, p, ps);
    if ((uint64_t)nlayers * 20 > sc.size()) fail(MLEM_EIO, "Error reading scanner geometry configuration");
    p += 20ull * nlayers;
    rd<uint32_t>(sc, p, ps);  // nBlocks
    const uint32_t bsize = rd<uint32_t>(sc, p, ps);
    if (bsize == 0 || (uint64_t)(bsize - 1) * 4 > sc.size()) fail(MLEM_EIO, "Error reading scanner geometry configuration");
    p += 4ull * (bsize - 1);
    const uint32_t nrings = rd<uint32_t>(sc, p, ps);
    if (nrings == 0 || (uint64_t)(nrings - 1) * 4 > sc.size()) fail(MLEM_EIO, "Error reading scanner geometry configuration");
    p += 4ull * (nrings - 1);
    p += 12;  // voxel size
    info.h.nx = rd<uint32_t>(sc, p, ps);
    info.h.ny = rd<uint32_t>(sc, p, ps);
    info.h.nz = rd<uint32_t>(sc, p, ps);
    if (p != info.scan_bytes) fail(MLEM_EIO, "Error reading scanner geometry configuration");
    info.data_off = 28ull + info.scan_bytes + 8ull * info.h.rows;
    return info;
}

void write_exact(FILE* f, const void* src, uint64_t bytes, const std::string& what) {
    if (bytes && std::fwrite(src, 1, bytes, f) != bytes) fail(MLEM_EIO, "short write: " + what);
}

// {u32 column, f32 value} pairs (matrixelement.hpp:37-46) -> SoA idx/val;
// any column >= cols raises *err.
__global__ void k_csr4_split(const uint2* __restrict__ pairs, uint64_t n, uint32_t cols, uint32_t* __restrict__ idx,
                             uint32_t* __restrict__ val_bits, uint32_t* __restrict__ err) {
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
        const uint2 p = pairs[i];
        if (p.x >= cols) atomicOr(err, 1u);
        idx[i] = p.x;
        val_bits[i] = p.y;
    }
}

// Streams the csr4 file into the device CSR A: the row END offsets are read on
// the host and checked like mlem_csr4_read; the element pairs are read in
// chunks into two pinned staging buffers (the read of chunk i+1 overlaps the
// copy and the split of chunk i) and split on the GPU into the column and
// value arrays (the host AoS->SoA loop of csr_format_for_cuda, main.cu:518-554,
// moved to the device).
void csr4_ingest(const char* path, const Csr4Info& info, DevCsr& A, cudaStream_t s) {
    const uint32_t rows = info.h.rows;
    const uint64_t nnz = info.h.nnz;
    File fh(path, "rb");
    if (!fh.f) fail(MLEM_EIO, std::string("Cannot open file ") + path);
    if (fseeko(fh.f, (off_t)(28 + info.scan_bytes), SEEK_SET) != 0) fail(MLEM_EIO, "seek failed");
    std::vector<uint64_t> rp((uint64_t)rows + 1);
    rp[0] = 0;
    read_exact(fh.f, rp.data() + 1, 8ull * rows, "row indexes");
    for (uint32_t r = 0; r < rows; ++r)
        if (rp[r + 1] < rp[r]) fail(MLEM_EIO, "csr4: row offsets are not monotone");
    if (rows && rp[rows] != nnz) fail(MLEM_EIO, "csr4: last row offset differs from nnz");
    A.nrows = rows;
    A.ncols = info.h.cols;
    A.nnz = nnz;
    A.vt = MLEM_VAL_F32;
    MLEM_CUDA(cudaMalloc(&A.rowptr, sizeof(uint64_t) * ((uint64_t)rows + 1)));
    MLEM_CUDA(cudaMalloc(&A.idx, sizeof(uint32_t) * padded(nnz)));
    MLEM_CUDA(cudaMalloc(&A.val, sizeof(float) * padded(nnz)));
    if (padded(nnz) > nnz) {
        MLEM_CUDA(cudaMemsetAsync(A.idx + nnz, 0, sizeof(uint32_t) * (padded(nnz) - nnz), s));
        MLEM_CUDA(cudaMemsetAsync(static_cast<float*>(A.val) + nnz, 0, sizeof(float) * (padded(nnz) - nnz), s));
    }
    MLEM_CUDA(cudaMemcpyAsync(A.rowptr, rp.data(), sizeof(uint64_t) * ((uint64_t)rows + 1), cudaMemcpyHostToDevice,
                              s));
    const uint64_t chunk = std::min<uint64_t>(nnz ? nnz : 1, 1ull << 23);  // pairs per chunk (64 MiB)
    uint2* host[2] = {nullptr, nullptr};
    uint2* dev[2] = {nullptr, nullptr};
    cudaEvent_t done[2] = {nullptr, nullptr};
    uint32_t* err = nullptr;
    auto release = [&] {
        cudaStreamSynchronize(s);
        for (int k = 0; k < 2; ++k) {
            if (host[k]) cudaFreeHost(host[k]);
            if (dev[k]) cudaFree(dev[k]);
            if (done[k]) cudaEventDestroy(done[k]);
        }
        if (err) cudaFree(err);
    };
    try {
        MLEM_CUDA(cudaMalloc(&err, sizeof(uint32_t)));
        MLEM_CUDA(cudaMemsetAsync(err, 0, sizeof(uint32_t), s));
        for (int k = 0; k < 2 && nnz; ++k) {
            MLEM_CUDA(cudaMallocHost(&host[k], sizeof(uint2) * chunk));
            MLEM_CUDA(cudaMalloc(&dev[k], sizeof(uint2) * chunk));
            MLEM_CUDA(cudaEventCreateWithFlags(&done[k], cudaEventDisableTiming));
        }
        uint64_t i = 0;
        for (uint64_t e = 0; e < nnz; e += chunk, ++i) {
            const int k = (int)(i & 1);
            const uint64_t n = std::min(chunk, nnz - e);
            if (i >= 2) MLEM_CUDA(cudaEventSynchronize(done[k]));  // staging k free again
            read_exact(fh.f, host[k], 8 * n, "matrix elements");
            MLEM_CUDA(cudaMemcpyAsync(dev[k], host[k], 8 * n, cudaMemcpyHostToDevice, s));
            const unsigned grid = std::max(1u, std::min<unsigned>(ceil_div_u(n, 256), 152u * 16u));
            k_csr4_split<<<grid, 256, 0, s>>>(dev[k], n, info.h.cols, A.idx + e,
                                              reinterpret_cast<uint32_t*>(A.val) + e, err);
            MLEM_LAUNCHED();
            MLEM_CUDA(cudaEventRecord(done[k], s));
        }
        uint32_t h = 0;
        MLEM_CUDA(cudaMemcpyAsync(&h, err, sizeof(uint32_t), cudaMemcpyDeviceToHost, s));
        MLEM_CUDA(cudaStreamSynchronize(s));
        if (h) fail(MLEM_EIO, "csr4: column index out of range");
    } catch (...) {
        release();
        throw;
    }
    release();
}

}  // namespace
}  // namespace mlem

using namespace mlem;

extern "C" {

mlem_status mlem_csr4_read_header(const char* path, mlem_csr4_header* hdr) {
    return guarded([&] {
        MLEM_REQUIRE(path && hdr, MLEM_EINVAL, "NULL argument");
        *hdr = parse_header(path).h;
    });
}

mlem_status mlem_csr4_read(const char* path, uint64_t* rowptr, uint32_t* col, float* val) {
    return guarded([&] {
        MLEM_REQUIRE(path && rowptr, MLEM_EINVAL, "NULL argument");
        const Csr4Info info = parse_header(path);
        const uint32_t rows = info.h.rows;
        const uint64_t nnz = info.h.nnz;
        MLEM_REQUIRE(nnz == 0 || (col && val), MLEM_EINVAL, "NULL argument");
        File fh(path, "rb");
        if (!fh.f) fail(MLEM_EIO, std::string("Cannot open file ") + path);
        std::fseek(fh.f, (long)(28 + info.scan_bytes), SEEK_SET);
        rowptr[0] = 0;
        read_exact(fh.f, rowptr + 1, 8ull * rows, "row indexes");
        for (uint32_t r = 0; r < rows; ++r)
            if (rowptr[r + 1] < rowptr[r]) fail(MLEM_EIO, "csr4: row offsets are not monotone");
        if (rows && rowptr[rows] != nnz) fail(MLEM_EIO, "csr4: last row offset differs from nnz");
        const uint64_t chunk = 1ull << 22;
        std::vector<uint32_t> buf(2 * chunk);
        for (uint64_t e = 0; e < nnz; e += chunk) {
            const uint64_t n = std::min(chunk, nnz - e);
            read_exact(fh.f, buf.data(), 8 * n, "matrix elements");
            for (uint64_t k = 0; k < n; ++k) {
                const uint32_t c = buf[2 * k];
                if (c >= info.h.cols) fail(MLEM_EIO, "csr4: column index out of range");
                col[e + k] = c;
                std::memcpy(val + e + k, &buf[2 * k + 1], 4);
            }
        }
    });
}

mlem_status mlem_csr4_write(const char* path, const mlem_csr4_scanner* sc, const mlem_csr_host* csr) {
    return guarded([&] {
        MLEM_REQUIRE(path && sc && csr && csr->rowptr, MLEM_EINVAL, "NULL argument");
        MLEM_REQUIRE(sc->n_layers >= 1 && sc->block_size >= 1 && sc->n_rings >= 1, MLEM_EINVAL,
                     "scanner needs at least one layer, block element and ring");
        MLEM_REQUIRE(csr->rowptr[0] == 0 && csr->rowptr[csr->rows] == csr->nnz, MLEM_EINVAL, "bad rowptr");
        File fh(path, "wb");
        if (!fh.f) fail(MLEM_EIO, std::string("Cannot open file ") + path);
        const uint32_t scan_bytes = 4 + 20 * sc->n_layers + 8 + 4 * (sc->block_size - 1) + 4 +
                                    4 * (sc->n_rings - 1) + 12 + 12;
        unsigned char hdr[28] = {'P', 'C', 'S', 'R', 4, sc->sym_flags, 0, 0};
        std::memcpy(hdr + 8, &csr->rows, 4);
        std::memcpy(hdr + 12, &csr->cols, 4);
        std::memcpy(hdr + 16, &csr->nnz, 8);
        std::memcpy(hdr + 24, &scan_bytes, 4);
        write_exact(fh.f, hdr, 28, path);
        std::vector<unsigned char> b;
        auto put = [&](const void* p, size_t n) {
            const unsigned char* c = static_cast<const unsigned char*>(p);
            b.insert(b.end(), c, c + n);
        };
        put(&sc->n_layers, 4);
        for (uint32_t l = 0; l < sc->n_layers; ++l) {
            const float lay[5] = {sc->crystal_w, sc->crystal_h, sc->crystal_d, sc->radius, sc->mu};
            put(lay, 20);
        }
        put(&sc->n_blocks, 4);
        put(&sc->block_size, 4);
        for (uint32_t i = 0; i + 1 < sc->block_size; ++i) put(&sc->block_gap, 4);
        put(&sc->n_rings, 4);
        for (uint32_t i = 0; i + 1 < sc->n_rings; ++i) put(&sc->ring_gap, 4);
        const float vs[3] = {sc->voxel_w, sc->voxel_h, sc->voxel_d};
        put(vs, 12);
        const uint32_t dims[3] = {sc->nx, sc->ny, sc->nz};
        put(dims, 12);
        MLEM_REQUIRE(b.size() == scan_bytes, MLEM_EINVAL, "internal: scanner config size");
        write_exact(fh.f, b.data(), b.size(), path);
        write_exact(fh.f, csr->rowptr + 1, 8ull * csr->rows, path);
        const uint64_t chunk = 1ull << 22;
        std::vector<uint32_t> buf(2 * chunk);
        for (uint64_t e = 0; e < csr->nnz; e += chunk) {
            const uint64_t n = std::min(chunk, csr->nnz - e);
            for (uint64_t k = 0; k < n; ++k) {
                buf[2 * k] = csr->col[e + k];
                std::memcpy(&buf[2 * k + 1], csr->val + e + k, 4);
            }
            write_exact(fh.f, buf.data(), 8 * n, path);
        }
    });
}

mlem_status mlem_matrix_load_csr4(const char* path, const mlem_matrix_opts* opts, mlem_matrix** out) {
    return guarded([&] {
        MLEM_REQUIRE(path && out, MLEM_EINVAL, "NULL argument");
        *out = nullptr;
        mlem_matrix_opts o;
        mlem_matrix_opts_default(&o);
        if (opts) o = *opts;
        const Csr4Info info = parse_header(path);
        MLEM_REQUIRE(info.h.rows >= 1 && info.h.cols >= 1, MLEM_EINVAL, "matrix must have rows and columns");
        if (o.layout != MLEM_LAYOUT_NATURAL && o.grid_nx == 0) {  // the file's scanner configuration
            o.grid_nx = info.h.nx;
            o.grid_ny = info.h.ny;
            o.grid_nz = info.h.nz;
        }
        *out = create_matrix_filled(o, [&](mlem_matrix* m) { csr4_ingest(path, info, m->A, m->stream); });
    });
}

mlem_status mlem_read_sinogram(const char* path, int32_t* g, uint64_t capacity, uint64_t* count_out) {
    return guarded([&] {
        MLEM_REQUIRE(path, MLEM_EINVAL, "NULL argument");
        File fh(path, "rb");
        if (!fh.f) fail(MLEM_EIO, std::string("Cannot open file ") + path);
        const uint64_t size = file_size(fh.f);
        if (size % 4 != 0) fail(MLEM_EIO, std::string("Cannot open file ") + path);
        const uint64_t n = size / 4;
        if (count_out) *count_out = n;
        if (!g) return;
        MLEM_REQUIRE(n <= capacity, MLEM_EINVAL, "sinogram larger than the buffer");
        read_exact(fh.f, g, size, path);
    });
}

mlem_status mlem_write_image(const char* path, const float* f, uint64_t count) {
    return guarded([&] {
        MLEM_REQUIRE(path && (f || count == 0), MLEM_EINVAL, "NULL argument");
        File fh(path, "wb");
        if (!fh.f) fail(MLEM_EIO, std::string("Cannot open file ") + path);
        write_exact(fh.f, f, 4 * count, path);
    });
}

uint64_t mlem_siddon_rows(const mlem_geometry* geo) {
    uint64_t n = 0;
    guarded([&] { n = geo ? siddon_rows(*geo) : 0; });
    return n;
}

mlem_status mlem_siddon_count_host(const mlem_geometry* geo, uint64_t* rowptr_out) {
    return guarded([&] {
        MLEM_REQUIRE(geo && rowptr_out, MLEM_EINVAL, "NULL argument");
        siddon_count_host(*geo, rowptr_out);
    });
}

mlem_status mlem_siddon_fill_host(const mlem_geometry* geo, const uint64_t* rowptr, uint32_t* col, float* val) {
    return guarded([&] {
        MLEM_REQUIRE(geo && rowptr && col && val, MLEM_EINVAL, "NULL argument");
        siddon_fill_host(*geo, rowptr, col, val);
    });
}

}  // extern "C"
