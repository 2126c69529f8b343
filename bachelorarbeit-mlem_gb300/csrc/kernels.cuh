// kernels.cuh — launchers of the device kernels (one declaration per kernel
// family; definitions in spmv.cu, merge.cu, transpose.cu, siddon.cu, batch.cu).
#pragma once

#include "common.cuh"

#include <algorithm>
#include <vector>

namespace mlem {

// L2 persisting window for the gathered vector of one launch (0 bytes = none).
struct L2Window {
    const void* ptr = nullptr;
    size_t bytes = 0;
};

// ------------------------------------------------------------- spmv.cu
// Epilogue selection for the row-wise products.
enum class Epi : int {
    Correl = 0,   // out[r] = sum != 0 ? g[r] / sum : 0   (calcCorrel, kernel.cu:11-19)
    Update = 1,   // f[c] = f[c]*sum/norm[c] (or f*sum if norm==0) (calcUpdate, kernel.cu:28-39)
    Raw = 2       // out[r] = sum
};

struct EpiArgs {
    Epi kind = Epi::Raw;
    const int32_t* g = nullptr;   // Correl
    float* out = nullptr;         // Correl: ratio; Raw: result
    float* fwproj = nullptr;      // Correl: optional copy of the projection
    float* f = nullptr;           // Update: image, updated in place
    const float* norm = nullptr;  // Update
    // symmetry-compressed kernels only: also write the results in orbit
    // order (Correl: ratio into SymOps::orb_r; Update: image into orb_x), and
    // take the input's orbit array as current instead of gathering it
    float* orbit_out = nullptr;
    bool orbit_ready = false;
    // ... and, inside an MLEM loop of two such projections, keep everything in
    // orbit order: g (Correl), the image and the sensitivity (Update) are read
    // from their orbit arrays and no natural-order output is written (fwproj
    // excepted)
    bool orbit_only = false;
};

// Rows of `op` times x, one group of `lanes` (4/8/16/32) threads per row,
// 128-bit loads of indices and values, deterministic reduction order.
// ordered: rows in op.order; pipelined: the next vectors are loaded before
// the current gathers (both for 16 or 32 lanes; same results).
void launch_csrvec(const DevCsr& op, const float* x, const EpiArgs& epi, int lanes,
                   L2Window win, cudaStream_t s, int unroll = 2, bool ordered = false, bool pipelined = false);
// Lane-interleaved copy (elements permuted inside 128-blocks) and its projection.
void build_ilv(DevCsr& op, cudaStream_t s);
void launch_csr_ilv(const DevCsr& op, const float* x, const EpiArgs& epi, int unroll, L2Window win,
                    cudaStream_t s);
// Delta-compressed (16-bit) column indices: build from the u32 indices, and
// the projection that reads them.
void build_d16(DevCsr& op, cudaStream_t s);
// unroll: 1 or 2 vectors of 8 entries in flight per lane (the lanes per row
// are those the layout was built for).
void launch_csr_d16(const DevCsr& op, const float* x, const EpiArgs& epi, int unroll, L2Window win, cudaStream_t s);
// Persistent, software-pipelined csr-vector variant (16 or 32 lanes per row,
// 1 or 2 vectors per lane and step, optional locality order); bit-identical
// to launch_csrvec with the same lanes.  prepare_* settles the grid sizes
// outside stream captures.
void prepare_csrvec_pipe(mlem_value_type vt);
void launch_csrvec_pipe(const DevCsr& op, const float* x, const EpiArgs& epi, int lanes, int unroll, bool ordered,
                        L2Window win, cudaStream_t s);
// Same product through the TMA-pipelined kernel (spmv_tma.cu); *err is set
// when a bounded wait expires.  prepare_* settles attributes outside captures.
void prepare_csr_tma(mlem_value_type vt);
void launch_csr_tma(const DevCsr& op, const float* x, const EpiArgs& epi, uint32_t* err, L2Window win,
                    cudaStream_t s);
// The scatter through per-warp shared-memory rings fed by cp.async.bulk
// (spmv_tma.cu); rows with ratio 0 are not read.  *err is set when a bounded
// wait expires; prepare_csr_tma settles its attributes outside captures.
void launch_scatter_tma(const DevCsr& A, const float* ratio, float* bp, uint32_t* err, L2Window win,
                        cudaStream_t s);
// bp[idx] += val * ratio[row] over the rows of A (calcBwProj_none_trans, kernel.cu:165-177);
// lanes per row 8/16/32, unroll = 16-byte vectors per lane in flight (1 or 2).
void launch_scatter(const DevCsr& A, const float* ratio, float* bp, int lanes, int unroll, L2Window win,
                    cudaStream_t s);
// One pass over A: sum = A[r,:]·x, ratio = g[r]/sum, bp[idx] += val*ratio.
void launch_fused_fp_scatter(const DevCsr& A, const float* x, const int32_t* g, float* bp,
                             float* fwproj, L2Window win, cudaStream_t s);
// The same pass by a group of `lanes` (8/16/32) per row that sums the row as
// launch_csrvec does (unroll 1 or 2 vectors in flight per lane), then
// re-walks it from L2 to scatter; ordered: rows in A.order.
void launch_fused_rescan(const DevCsr& A, const float* x, const int32_t* g, float* bp, float* fwproj, int lanes,
                         int unroll, bool ordered, L2Window win, cudaStream_t s);
// ------------------------------------------------------------- spmv_fused.cu
// The rows of A in chunks of whole rows for the staged fused pass: a chunk's
// span of entries, aligned to 8, fits one shared-memory stage and holds at
// most kFusedMaxRows rows; a row longer than a stage is a chunk of its own
// ("wide", read from global memory).  The stage is worked in blocks of
// kFusedBlk entries; a piece is the part of one row inside one block.
constexpr int kFusedCap = 4096;     // entries per stage
constexpr int kFusedMaxRows = 128;  // rows per chunk
constexpr int kFusedBlk = 128;      // entries per block (32 lanes x 4)
struct alignas(16) FusedChunk {
    uint64_t a0;        // first entry of the staged span (multiple of 8)
    uint64_t meta_off;  // the chunk's metadata in FusedPlan::meta (multiple of 4)
    uint32_t n8;        // staged span in 8-entry units
    uint32_t r0;        // first row
    uint16_t nr;        // rows
    uint16_t wide;      // 1: one row longer than a stage, not staged
    uint32_t mlen;      // metadata words: rs[nr+1], pf[nr+1], bf[nb] (wide: rs[2])
};
// Metadata of a chunk (u32, relative to a0): rs[j] = start of row j (rs[nr]
// = end of the last row); pf[j] = index of row j's first piece in the chunk's
// piece order (pf[nr] = pieces); bf[b] = first row that ends after block b
// starts (nb = blocks up to rs[nr]).
struct FusedPlan {
    uint64_t nchunks = 0;
    FusedChunk* chunks = nullptr;  // [nchunks]
    uint32_t* meta = nullptr;      // [meta_len]
    uint64_t meta_len = 0;
    bool built = false;
    int staged_threads = 0;        // timed CTA size of the staged kernel (256 or 512; 0 = not yet)
    float staged_ms = 0.f;         // and its time for one pass
    void release();
};
// A form of the fused single pass.
struct FusedForm {
    int kind = 0;          // 0 register (k_fused), 1 staged (k_fused_staged), 2 rescan (k_fused_rescan)
    int threads = 256;     // staged: CTA size
    int lanes = 16;        // rescan: lanes per row
    int unroll = 2;        // rescan: vectors per lane in flight
    bool ordered = false;  // rescan: rows in locality order
    float ms = 0.f;        // measured time of one pass
};
// Cuts the rows of A into chunks (host pass over the row pointers, once).
void fused_plan_build(const DevCsr& A, FusedPlan& p, cudaStream_t s);
// Kernel attributes and grid sizes, settled outside stream captures.
void prepare_fused_staged(mlem_value_type vt);
// The staged single pass: same results as launch_fused_fp_scatter up to the
// order of the FP32 additions (products rounded before the row sum; the
// scatter's atomic order is unordered in both).  *err is set when a bounded
// wait expires.
void launch_fused_staged(const DevCsr& A, const FusedPlan& p, int threads, const float* x, const int32_t* g,
                         float* bp, float* fwproj, uint32_t* err, L2Window win, cudaStream_t s);
// f = f*bp/norm (or f*bp), then bp = 0 — update of the scatter forms.
void launch_update_zero(float* f, float* bp, const float* norm, uint32_t n, cudaStream_t s);
// Σ_r g_r log(fp_r) - fp_r over rows with fp_r > 0, FP64, fixed reduction order.
void launch_loglik(const int32_t* g, const float* fwproj, uint32_t rows, double* part,
                   double* out, cudaStream_t s);
constexpr int kLoglikParts = 1024;
int pick_lanes(uint64_t nnz, uint32_t rows);

// ------------------------------------------------------------- merge.cu
// Reference partition search for thread starts t*secsize (kernel.cu:190-241).
void launch_merge_search_ref(const uint64_t* rowptr, uint32_t rows, uint64_t nnz,
                             uint32_t secsize, uint64_t nthreads, int64_t* i_out,
                             int64_t* j_out, cudaStream_t s);

struct MergePlan {
    uint32_t secsize = 0;
    uint32_t threads = 0;   // threads per CTA
    uint64_t ntiles = 0;
    uint32_t* tile_i = nullptr;   // [ntiles+1]
    uint64_t* tile_j = nullptr;   // [ntiles+1]
    float* carry = nullptr;       // [ntiles]
    uint32_t* carry_row = nullptr;// [ntiles]
    float* head = nullptr;        // [ntiles]
    size_t smem = 0;
    // true: the row-parallel tile kernel (library-owned, padded operands);
    // false: the per-thread walk over shared-memory products (any arrays)
    bool rows_kernel = false;
    int rows_u = 1;              // row kernel: vectors per lane in flight (1: 8 blocks per SM, 2: 6)
    void release();
};
// Builds the tile partition of `op` for a section size (device allocations).
void merge_plan_build(const DevCsr& op, uint32_t secsize, MergePlan& plan, cudaStream_t s);
// Merge-path product with deterministic carry fix-up (2 launches).
void launch_merge_spmv(const DevCsr& op, const MergePlan& plan, const float* x,
                       const EpiArgs& epi, L2Window win, cudaStream_t s);

// ------------------------------------------------------------- transpose.cu
// Stable counting sort by column of A (f32 values) -> Aᵀ with u32 row ids.
void transpose_device(const DevCsr& A, DevCsr& AT, cudaStream_t s);
// norm[c] = (float) Σ (double) val over column c.
void colsum_from_transpose(const DevCsr& AT, float* norm, cudaStream_t s);
void colsum_scatter(const DevCsr& A, float* norm, cudaStream_t s);
// Value conversion f32 -> f16/bf16 (n elements, padded tail included).
void convert_values(const float* src, void* dst, mlem_value_type vt, uint64_t n, cudaStream_t s);
void convert_values_back(const void* src, float* dst, mlem_value_type vt, uint64_t n,
                         cudaStream_t s);
uint32_t max_row_length(const uint64_t* rowptr, uint32_t rows, cudaStream_t s);
// Exclusive scan of u32 counts into u64 offsets; out[n] = total.
void scan_counts_u64(const uint32_t* in, uint64_t* out, uint64_t n, cudaStream_t s);
// rowptr u64[rows+1] with leading zero; device copy sanity check (monotone, last == nnz,
// indices < cols).  Returns false when the CSR is malformed.
bool validate_csr(const DevCsr& A, cudaStream_t s);

// ------------------------------------------------------------- layout.cu
// out[k] = in[map[k]] (natural -> internal order) / out[map[k]] = in[k]
// (internal -> natural); map[k] = natural index of internal index k.
void launch_gather_i32(int32_t* out, const int32_t* in, const uint32_t* map, uint64_t n, cudaStream_t s);
void launch_gather_f32(float* out, const float* in, const uint32_t* map, uint64_t n, cudaStream_t s);
void launch_scatter_f32(float* out, const float* in, const uint32_t* map, uint64_t n, cudaStream_t s);
// inv[map[k]] = k
void launch_invert_perm(const uint32_t* map, uint32_t n, uint32_t* inv, cudaStream_t s);
// out row k = in row row_src[k] (NULL: k) with columns c -> col_map[c] (NULL:
// unchanged), sorted; *keep_t (optional) receives the transpose of out.  f32.
void remap_csr(const DevCsr& in, const uint32_t* row_src, const uint32_t* col_map, DevCsr& out, DevCsr* keep_t,
               cudaStream_t s);
// Row order of a matrix without a detector numbering: rows sorted (stably) by
// the coarse voxel cells of their lowest and highest column, empty rows last.
// Returns the natural row of every internal row.
std::vector<uint32_t> derived_lor_order(const DevCsr& A, uint32_t nx, uint32_t ny, uint32_t nz, cudaStream_t s);

// ------------------------------------------------------------- symmetry.cu
// Symmetry-compressed projection operands of a generated cylindrical scanner
// (see symmetry.cu).  Rows: canonical LORs (forward projection) and canonical
// voxels (back projection over A^T); an entry names its column as an orbit
// row and a transformation, key = orbit << 4 | t.  The orbit arrays hold the
// input vector in orbit order (16 floats per canonical voxel / LOR) and are
// per-handle scratch, refilled before every projection.
struct SymOps {
    uint32_t K = 0, J = 0;           // canonical LOR rows / canonical voxel rows
    uint64_t fp_nnz = 0, bp_nnz = 0;
    uint64_t* fp_rowptr = nullptr;   // [4 K + 1] row k, segment q (entries with t & 3 == q): 4 k + q
    uint32_t* fp_key = nullptr;      // [fp_nnz] canonical voxel << 4 | t
    void* fp_val = nullptr;          // [fp_nnz]
    uint32_t* img = nullptr;         // [16 K] LOR s(r_k)
    uint64_t* lead = nullptr;        // [K] 4 bits per s: first transformation with the same LOR
    uint64_t* bp_rowptr = nullptr;   // [4 J + 1]
    uint32_t* bp_key = nullptr;      // [bp_nnz] canonical LOR << 4 | t
    void* bp_val = nullptr;          // [bp_nnz]
    uint32_t* vimg = nullptr;        // [16 J] voxel s(v_j)
    uint64_t* vlead = nullptr;       // [J] 4 bits per s: first transformation with the same voxel
    float* orb_x = nullptr;          // [16 J] image in orbit order (forward projection input)
    float* orb_r = nullptr;          // [16 K] ratio in orbit order (back projection input)
    float* norm_orb = nullptr;       // [16 J] sensitivity image in orbit order
    int32_t* g_orb = nullptr;        // [16 K] sinogram of the running reconstruction in orbit order
    mlem_value_type vt = MLEM_VAL_F32;
    void release();
    uint64_t bytes() const;
};
// Geometry requirements of the symmetric form (errors otherwise).
void check_symmetric_geometry(const mlem_geometry& geo);
// A^ (symmetrised from the canonical rows), its transpose, and the compact
// operands; A and AT must be empty.
void build_symmetric(const mlem_geometry& geo, DevCsr& A, DevCsr& AT, SymOps& y, cudaStream_t s);
// The same from a caller's matrix (host CSR c, already uploaded as `user`):
// its rows must be the D(D-1)/2 detector pairs of a ring scanner with dpr
// detectors per ring and `rings` rings, its columns an n x n x nz grid.  A^ is
// built from the canonical rows of c and must equal `user` bit for bit (the
// matrix is invariant under the 16 transformations); otherwise MLEM_EINVAL.
// A, AT and y are filled either way and owned by the caller.
void build_symmetric_checked(const mlem_csr_host& c, const DevCsr& user, uint32_t n, uint32_t nz, uint32_t dpr,
                             uint32_t rings, DevCsr& A, DevCsr& AT, SymOps& y, cudaStream_t s);
void lower_symmetric_values(SymOps& y, mlem_value_type vt, cudaStream_t s);
// Forward (transposed = false: Correl or Raw epilogue) or back projection
// (true: Update or Raw) through the compact operands; natural order in and out.
// Orbit arrays of the sensitivity image (once per matrix), of the image and
// of the sinogram (at the start of an MLEM loop), and the image back in
// natural order (at its end).
void sym_set_norm(SymOps& y, const float* norm, cudaStream_t s);
void sym_gather_image(const SymOps& y, const float* f, cudaStream_t s);
void sym_gather_sinogram(const SymOps& y, const int32_t* g, cudaStream_t s);
void sym_scatter_image(const SymOps& y, float* f, cudaStream_t s);
// unroll: entries per lane in flight (2, 4 or 8); grouped: the blocks that
// start together on an SM take neighbouring rows.
void launch_sym(const SymOps& y, bool transposed, const float* x, const EpiArgs& e, int unroll, bool grouped,
                L2Window win, cudaStream_t s);

// ------------------------------------------------------------- siddon.cu
uint64_t siddon_rows(const mlem_geometry& geo);
void siddon_count_host(const mlem_geometry& geo, uint64_t* rowptr);
void siddon_fill_host(const mlem_geometry& geo, const uint64_t* rowptr, uint32_t* col, float* val);
void siddon_generate_device(const mlem_geometry& geo, DevCsr& A, cudaStream_t s);
// Rows of the given LOR indices (row_stride 1), generated on the host.
void siddon_rows_of_lors(const mlem_geometry& geo, const std::vector<uint64_t>& lors, std::vector<uint64_t>& rowptr,
                         std::vector<uint32_t>& col, std::vector<float>& val);
// Locality-friendly processing orders for a generated matrix: LORs in 4x4
// detector tubes (rows of A) and voxels in 4x2x2 bricks (rows of Aᵀ).
std::vector<uint32_t> siddon_lor_order(const mlem_geometry& geo);
std::vector<uint32_t> voxel_brick_order(uint32_t nx, uint32_t ny, uint32_t nz, uint32_t bx = 4, uint32_t by = 2,
                                        uint32_t bz = 2);

// ------------------------------------------------------------- batch.cu
// Interleaved batch state: slot b of voxel c is f[c*tile + b]; g and ratio
// are [rows][tile]; remaining[b] counts the iterations slot b still runs.
struct BatchArgs {
    uint32_t tile = 16;          // instances per tile (8/16/32)
    uint32_t active = 0;         // slots 0..active-1 may have iterations left (0 = the whole tile)
    const int32_t* g = nullptr;
    float* f = nullptr;
    float* ratio = nullptr;
    uint32_t* remaining = nullptr;
    // slots the projections cover: the smallest power of two >= active, 4..tile
    uint32_t width() const {
        const uint32_t a = active ? std::min(active, tile) : tile;
        uint32_t w = 4;
        while (w < a) w <<= 1;
        return w;
    }
};
// Slots the projections cover for `active` leading slots in a tile (4..tile).
inline uint32_t batch_width(uint32_t tile, uint32_t active) {
    BatchArgs a;
    a.tile = tile;
    a.active = active;
    return a.width();
}
// `steps` whole iterations of the tile (FP, BP + update, tick) in one
// persistent cooperative launch with grid-wide barriers; count (one word,
// zeroed here before the launch) carries the barriers, *err becomes 1 if a
// barrier wait ran out (the launch then ends early).  Needs Aᵀ.
void launch_batch_loop(const DevCsr& A, const DevCsr& AT, const float* norm, const BatchArgs& b, uint32_t steps,
                       unsigned* count, int* err, cudaStream_t s);
// ratio[r][b] = g[r][b] / (A f_b)[r] for the slots b < width().
void launch_batch_fp(const DevCsr& A, const BatchArgs& b, L2Window win, cudaStream_t s);
// f_b = f_b * (Aᵀ ratio_b) / norm for slots b < width() with remaining > 0.
void launch_batch_bp_update(const DevCsr& AT, const float* norm, const BatchArgs& b,
                            L2Window win, cudaStream_t s);
// remaining[b] -= 1 where positive.
void launch_batch_tick(const BatchArgs& b, cudaStream_t s);
// Scatter form (no Aᵀ): bp[c][b] += A[r,c] * ratio[r][b], then update + zero.
void launch_batch_scatter(const DevCsr& A, const BatchArgs& b, float* bp, cudaStream_t s);
void launch_batch_update_zero(const float* norm, uint32_t cols, const BatchArgs& b, float* bp,
                              cudaStream_t s);
// Slot b <- sinogram g (contiguous), image f0 (contiguous) or the constant init,
// and its iteration count; slot b -> contiguous image.
// lor_of / vox_of (may be NULL): natural index of each internal row / column
// of a matrix in the locality layout; g, f0 and out are in natural order.
void launch_slot_put(int32_t* G, float* F, uint32_t rows, uint32_t cols, uint32_t BT, uint32_t b,
                     const int32_t* g, float init, const float* f0, uint32_t* remaining,
                     uint32_t iters, const uint32_t* lor_of, const uint32_t* vox_of, cudaStream_t s);
void launch_slot_get(const float* F, uint32_t cols, uint32_t BT, uint32_t b, float* out,
                     const uint32_t* vox_of, cudaStream_t s);

}  // namespace mlem

namespace mlem {
// Largest access-policy window the device accepts (0 until queried).
extern size_t g_max_window_bytes;

// Launch through cudaLaunchKernelEx so the L2 access-policy window travels
// with the launch (and into a CUDA graph node when captured).
template <typename... KArgs, typename... Args>
inline void launch_ex(void (*kernel)(KArgs...), dim3 grid, dim3 block, size_t smem,
                      cudaStream_t s, L2Window win, Args... args) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = grid;
    cfg.blockDim = block;
    cfg.dynamicSmemBytes = smem;
    cfg.stream = s;
    cudaLaunchAttribute attr[1];
    unsigned n = 0;
    if (win.bytes && g_max_window_bytes) {
        attr[0].id = cudaLaunchAttributeAccessPolicyWindow;
        attr[0].val.accessPolicyWindow.base_ptr = const_cast<void*>(win.ptr);
        attr[0].val.accessPolicyWindow.num_bytes = win.bytes < g_max_window_bytes ? win.bytes : g_max_window_bytes;
        attr[0].val.accessPolicyWindow.hitRatio = 1.0f;
        attr[0].val.accessPolicyWindow.hitProp = cudaAccessPropertyPersisting;
        attr[0].val.accessPolicyWindow.missProp = cudaAccessPropertyStreaming;
        n = 1;
    }
    cfg.attrs = attr;
    cfg.numAttrs = n;
    MLEM_CUDA(cudaLaunchKernelEx(&cfg, kernel, static_cast<KArgs>(args)...));
    count_launch();
}
}  // namespace mlem
