/*
 * mlem.h — C ABI of the GB300-native MLEM reconstructor.
 *
 * Drop-in for the single-device MLEM loop of wmd0701/Bachelorarbeit-MLEM.
 * Every entry point returns an mlem_status; mlem_last_error() gives the text
 * of the last failure on the calling thread.  Host buffers are owned by the
 * caller and never mutated unless they are documented outputs.  Device memory
 * is owned by the library through opaque handles.  A handle is used by one
 * host thread at a time (the server object is internally threaded).
 *
 * Reference interfaces replaced (file:line in the reference project):
 *   - mlem()                       main.cu:19, main.cu:167-514
 *   - main() argv contract         main.cu:42-62, help() main.cu:614-625
 *   - csr_format_for_cuda()        main.cu:518-554
 *   - calcColumnSums()             main.cu:558-580
 *   - partitionMatrix()            main.cu:593-611
 *   - sptrans_scanTrans_specialized sptrans.h:397-545
 *   - merge_based_start()          kernel.cu:190-241 (partition search)
 *   - Csr4Matrix(path)             helper_files_common/csr4matrix.cpp:36-178
 *   - Vector<int>(path), writeToFile helper_files_common/vector.hpp:33-87
 */
#ifndef MLEM_GB300_H
#define MLEM_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ------------------------------------------------------------------ status */
typedef enum {
    MLEM_OK = 0,
    MLEM_EINVAL = 1,      /* bad argument (the reference prints help() and exits) */
    MLEM_EIO = 2,         /* unreadable / malformed file (reference: runtime_error) */
    MLEM_ENOMEM = 3,      /* device or host allocation failed, or admission refused */
    MLEM_ECUDA = 4,       /* a CUDA runtime call failed */
    MLEM_ETIMEOUT = 5,    /* a bounded wait expired (server, persistent or staged kernels) */
    MLEM_EUNSUPPORTED = 6,/* size or mode outside what the library handles */
    MLEM_EBUSY = 7        /* server queue full / object in use */
} mlem_status;

/* Text of the last error raised on the calling thread ("" if none). */
const char* mlem_last_error(void);
/* Library version string. */
const char* mlem_version(void);

/* --------------------------------------------------------------- switches */
/* argv[8] of the reference CLI: 0 merge-based SpMV, 1 csr-vector SpMV. */
typedef enum { MLEM_SPMV_MERGE = 0, MLEM_SPMV_CSR_VECTOR = 1 } mlem_spmv;

/* Storage type of the matrix values on the device (accumulation is FP32). */
typedef enum { MLEM_VAL_F32 = 0, MLEM_VAL_F16 = 1, MLEM_VAL_BF16 = 2 } mlem_value_type;

/* Back-projection form.  MLEM_BP_TRANS and MLEM_BP_SCATTER are argv[7]=0 and
 * argv[7]=1 of the reference; MLEM_BP_FUSED is a single pass over A that does
 * forward projection, correlation and the scatter back projection row by row
 * (reads the matrix once per iteration; same operations as SCATTER, the
 * staged form rounds each product before the row sum). */
typedef enum { MLEM_BP_TRANS = 0, MLEM_BP_SCATTER = 1, MLEM_BP_FUSED = 2 } mlem_bp_mode;

/* ------------------------------------------------------------ host CSR */
/* SoA CSR as produced by csr_format_for_cuda (main.cu:518-554):
 * rowptr u64[rows+1] with rowptr[0] = 0, col u32[nnz], val f32[nnz]. */
typedef struct {
    uint32_t rows;
    uint32_t cols;
    uint64_t nnz;
    const uint64_t* rowptr;
    const uint32_t* col;
    const float* val;
} mlem_csr_host;

/* ------------------------------------------------------------- matrix */
typedef struct mlem_matrix mlem_matrix;

typedef struct {
    mlem_value_type value_type; /* device storage of values (F32 = plain method) */
    uint32_t build_transpose;   /* 1: build Aᵀ on the GPU (stable counting sort) */
    const float* norm;          /* optional host sensitivity image f32[cols];
                                   NULL = computed on the GPU as Aᵀ1 in FP64 */
    int device;                 /* CUDA device ordinal (reference: GPU 0) */
    uint32_t compress_indices;  /* 1: also keep a copy with 16-bit delta-coded column indices
                                   (each entry: the difference to the column 4 or 8 entries
                                   earlier in its row, plus its value; ~2.2 B of index per
                                   nonzero instead of 4, dummies and padding included) for the
                                   csr-vector projections (kernel D16, an autotuner candidate);
                                   with FP16 values the fastest form for a stored matrix */
    uint32_t interleave;        /* 1: also keep a lane-interleaved copy (16-byte loads whose
                                   gathers cover consecutive columns) for the projections */
    uint32_t layout;            /* mlem_layout: device order of rows and columns */
    uint32_t grid_nx, grid_ny, grid_nz; /* voxel grid of the columns (column = x + nx*(y + ny*z),
                                   scannerconfig.cpp:30-35) for the locality layout of
                                   mlem_matrix_create; csr4 files and geometries carry their own */
    uint32_t symmetry;          /* 1 = use the 16 symmetries of the scanner (mirror y -> -y, rotations
                                   by 90 degrees, axial flip) through compact operands holding 1/16 of
                                   the nonzeros for the csr-vector projections (kernel SYM, an
                                   autotuner candidate); natural layout only.
                                   mlem_matrix_generate (needs det_per_ring % 4 == 0, nx == ny,
                                   vx == vy, row_stride 1): the matrix becomes A^, built from the
                                   canonical LOR rows (averaged over the symmetries that fix their
                                   LOR) so that it is exactly symmetric; it stays the matrix of every
                                   mode and getter.
                                   mlem_matrix_create: the caller's matrix is kept unchanged; its rows
                                   must be the detector pairs (a < b, lexicographic; detector
                                   ring * sym_det_per_ring + k at angle 2 pi k / sym_det_per_ring) of
                                   a ring scanner, its columns the grid_nx x grid_nx x grid_nz voxels
                                   of a grid centred on the axis, and it must be exactly invariant
                                   under the 16 transformations (checked bit for bit against the
                                   symmetric matrix rebuilt from its canonical rows; MLEM_EINVAL
                                   otherwise).  No counterpart in the reference (its csr4 symmetry
                                   flags are not expanded, csr4matrix.cpp:72-75). */
    uint32_t sym_det_per_ring;  /* mlem_matrix_create with symmetry: detectors per ring (multiple of 4) */
    uint32_t sym_rings;         /* mlem_matrix_create with symmetry: rings */
} mlem_matrix_opts;

/* Device layout of a matrix.  LOCALITY stores A' = P_L A P_Vᵀ: columns
 * (voxels) in 4x4x2 bricks, rows (LORs) in 4x4 detector tubes for generated
 * matrices (other matrices: rows sorted by the coarse voxel cells of their
 * lowest and highest column), each row's columns ascending.  The
 * gathers of both projections then hit fewer cache lines.  Every entry point
 * still takes and returns natural order (sinograms, images, projections,
 * mlem_matrix_get_csr / _transpose / _norm); results agree with the natural
 * layout to FP32 rounding (the order of each row's additions changes). */
typedef enum { MLEM_LAYOUT_NATURAL = 0, MLEM_LAYOUT_LOCALITY = 1 } mlem_layout;

/* Fills *o with the defaults: F32 values, transpose built, norm computed, device 0. */
void mlem_matrix_opts_default(mlem_matrix_opts* o);

/* Uploads A (host CSR), optionally builds Aᵀ and the sensitivity image on the
 * device.  Replaces the H2D part of mlem() (main.cu:236-299), the host
 * transpose (main.cu:100-105) and calcColumnSums (main.cu:558-580). */
mlem_status mlem_matrix_create(const mlem_csr_host* csr, const mlem_matrix_opts* opts,
                               mlem_matrix** out);

/* Reads a csr4 file (helper_files_common/csr4matrix.cpp:36-178 format) and
 * creates the device matrix from it: the row offsets are read and checked on
 * the host, the {column, value} pairs stream through pinned staging buffers
 * and are split into the device CSR arrays on the GPU (replaces Csr4Matrix +
 * csr_format_for_cuda, main.cu:76-79, 518-554).  Malformed files fail with
 * MLEM_EIO, as mlem_csr4_read. */
mlem_status mlem_matrix_load_csr4(const char* path, const mlem_matrix_opts* opts,
                                  mlem_matrix** out);

mlem_status mlem_matrix_destroy(mlem_matrix* m);

typedef struct {
    uint32_t rows, cols;
    uint64_t nnz;
    mlem_value_type value_type;
    uint32_t has_transpose;
    uint64_t device_bytes;      /* bytes of device memory held by the handle */
    uint32_t max_row_nnz, max_col_nnz;
    /* symmetry = 1 only (else 0): canonical LOR rows and canonical voxels (the
     * rows of the two compact operands) and the entries of each operand */
    uint32_t sym_lor_rows, sym_voxel_rows;
    uint64_t sym_fp_nnz, sym_bp_nnz;
    /* compress_indices = 1 only (else 0): stored entries of the D16 copies of
     * A and of Aᵀ (nonzeros + dummies + padding; 2 bytes of index and one
     * value each) and the lanes per row their layout is built for */
    uint64_t d16_slots, d16_slots_t;
    uint32_t d16_lanes, d16_lanes_t;
} mlem_matrix_info;

mlem_status mlem_matrix_get_info(const mlem_matrix* m, mlem_matrix_info* info);
/* Configuration the autotuner chose for the csr-vector projection of A
 * (transposed = 0) or Aᵀ (1): kernel (mlem_kernel), lanes per row, vectors in
 * flight per lane, whether rows run in locality order, whether the row's
 * vector loads are software-pipelined, and the measured
 * milliseconds of one launch.  Tunes on first call if needed.
 * transposed = 2: the fused single pass (bp_mode 2) the AUTO switch picks —
 * kernel = the switch that selects that form (TMA staged, PERSISTENT
 * register, DIRECT / ordered rescan), lanes = lanes per row (staged: threads
 * per CTA), unroll and ordered as for the rescan form. */
mlem_status mlem_matrix_get_tuning(mlem_matrix* m, uint32_t transposed, int* kernel, int* lanes,
                                   int* unroll, int* ordered, int* pipelined, float* ms);
/* Copies the sensitivity image (f32[cols]) to the host. */
mlem_status mlem_matrix_get_norm(const mlem_matrix* m, float* norm_out);
/* Copies the device-built transpose to the host: colptr u64[cols+1],
 * rowidx u32[nnz], val f32[nnz] (same layout as sptrans_scanTrans_specialized
 * outputs cscColPtr / cscRowIdx / cscVal, sptrans.h:397-405). */
mlem_status mlem_matrix_get_transpose(const mlem_matrix* m, uint64_t* colptr,
                                      uint32_t* rowidx, float* val);

/* ------------------------------------------------------------------ run */
typedef struct {
    mlem_spmv spmv;             /* argv[8] */
    mlem_bp_mode bp_mode;       /* argv[7] (0 trans, 1 scatter) or 2 fused */
    uint32_t secsize_fp;        /* argv[5]: items per thread, merge FP, 1..512 */
    uint32_t secsize_bp;        /* argv[6]: items per thread, merge BP, 1..512 */
    uint32_t use_graph;         /* 1: replay the iteration as a CUDA graph */
    uint32_t loglik_every;      /* 0: off; k: FP64 log-likelihood every k-th iteration */
    uint32_t l2_window;         /* 1: keep the image/ratio vector L2-persisting */
    uint32_t kernel;            /* csr-vector switch: mlem_kernel variant (scatter mode: TMA
                                   also streams the scatter through shared-memory rings,
                                   AUTO takes it where it timed faster).  Fused pass
                                   (bp_mode 2): TMA = chunks staged through shared memory,
                                   PERSISTENT = one warp per row kept in registers, AUTO =
                                   the fastest form and configuration (timed once per
                                   matrix), any other = a group of `lanes` per row that
                                   re-walks its row from L2 for the scatter (`unroll`,
                                   ORDERED / row_order as for the projection) */
    uint32_t lanes;             /* DIRECT / PERSISTENT / ORDERED: lanes per row (4, 8, 16, 32;
                                   PERSISTENT 16 or 32); 0 = chosen from the mean row length */
    uint32_t unroll;            /* same kernels: vectors of 4 elements in flight per lane
                                   (1, 2, 4; PERSISTENT 1 or 2); 0 = 2.  SYM: entries in flight
                                   per lane, 2 (1, 2), 4 or 8 (0, 8).  D16: vectors of 8
                                   entries in flight per lane, 1 or 2 (0, 2) */
    uint32_t row_order;         /* DIRECT / PERSISTENT with 16 or 32 lanes: 1 = process the rows in
                                   the locality order of a generated matrix; SYM: 1 = the blocks that
                                   start together on an SM take neighbouring canonical rows */
    uint32_t pipeline;          /* DIRECT / ORDERED with 16 or 32 lanes: 1 = load a row's next vectors
                                   before the gathers of the current ones (same results) */
    uint32_t kernel_timing;     /* mlem_run only: 1 = CUDA events around the forward and back
                                   projection stages of every iteration (eager launches, no graph
                                   replay); their means go to mlem_stats.fp_ms / bp_ms */
    double loglik_rel_tol;      /* mlem_run with loglik_every > 0: 0 = run every iteration; t > 0 =
                                   convergence stop: the run ends after the first evaluated
                                   iteration whose log-likelihood gained less than t * |L| over the
                                   previous evaluation (the host reads each evaluation back);
                                   mlem_stats.iterations gives the iterations run, later
                                   loglik_out entries stay NaN.  No counterpart in the reference,
                                   which always runs argv[3] iterations. */
} mlem_run_opts;

/* Kernel variants of the csr-vector projections (same arithmetic; the order of
 * the FP32 additions depends on the variant and its lanes/unroll, so results of
 * different variants agree to rounding, and one matrix handle always uses one):
 *   DIRECT     one warp (or 4-32 lanes) per row, a grid of one row per group;
 *   PERSISTENT resident groups walk the rows, software-pipelined: the next
 *              step's index/value vectors (and the next row's pointers) are
 *              loaded before the current step's gathers;
 *   TMA        rows streamed into a shared-memory ring with cp.async.bulk. */
typedef enum {
    MLEM_KERNEL_DIRECT = 0,
    MLEM_KERNEL_TMA = 1,
    MLEM_KERNEL_PERSISTENT = 2,
    MLEM_KERNEL_AUTO = 3, /* autotuned per matrix operand (lanes per row, vectors in flight, variant) */
    MLEM_KERNEL_D16 = 4,  /* delta-coded indices (matrix created with compress_indices = 1) */
    MLEM_KERNEL_ILV = 5,  /* lane-interleaved copy (matrix created with interleave = 1) */
    MLEM_KERNEL_ORDERED = 6, /* DIRECT with rows in locality order (generated matrices:
                               LORs in 4x4 detector tubes, voxels in 4x2x2 bricks) */
    MLEM_KERNEL_SYM = 7   /* symmetry-compressed operands (generated with symmetry = 1) */
} mlem_kernel;

/* Defaults: CSR_VECTOR, BP_TRANS, secsize 5/5, graphs on, no log-likelihood, L2 window on,
 * AUTO kernel, lanes, unroll, row_order and pipeline 0. */
void mlem_run_opts_default(mlem_run_opts* o);

typedef struct {
    double seconds_total;       /* wall time of the call */
    double seconds_iterations;  /* device time of the iteration loop (CUDA events) */
    uint32_t iterations;
    uint32_t kernel_launches;   /* kernels launched by the iteration loop */
    uint64_t bytes_h2d, bytes_d2h;
    double loglik_last;         /* last computed log-likelihood (NaN if none) */
    double fp_ms, bp_ms;        /* mean forward / back projection stage (kernel_timing), else NaN */
} mlem_stats;

/* Runs `iterations` MLEM iterations on host buffers: g i32[rows] (sinogram),
 * f0 f32[cols] (NULL = reference initial value Σg/Σnorm, main.cu:83-97),
 * f_out f32[cols].  Replaces the loop and teardown of mlem() (main.cu:329-463).
 * loglik_out: optional f64[iterations] (NaN where not computed). */
mlem_status mlem_run(mlem_matrix* m, const int32_t* g, const float* f0, uint32_t iterations,
                     const mlem_run_opts* opts, float* f_out, double* loglik_out,
                     mlem_stats* stats);

/* Same loop on device buffers already resident in HBM: g_dev i32[rows],
 * f_dev f32[cols] holds f0 on entry and the image on exit.  Asynchronous on
 * `stream` (a cudaStream_t, NULL = legacy default stream).  A bounded wait
 * that expired inside a kernel of this call (TMA kernel, staged fused pass)
 * leaves a flag on the matrix that the next mlem_run reports as
 * MLEM_ETIMEOUT. */
mlem_status mlem_run_device(mlem_matrix* m, const int32_t* g_dev, float* f_dev,
                            uint32_t iterations, const mlem_run_opts* opts, void* stream);

/* Reference initial value: f0 = (float)Σg / Σnorm with Σnorm summed in FP32
 * in column order (main.cu:83-97). */
mlem_status mlem_initial_value(const mlem_matrix* m, const int32_t* g, float* init_out);

/* Drop-in with the exact argument list of the reference mlem() (main.cu:19):
 * host CSR of A (u64 row pointers), optional host CSR of Aᵀ (used when
 * using_trans == 0; if NULL the transpose is built on the GPU), g, norm,
 * f (initial image), result_f (output).  device_numbers must be 1.
 * Unlike the reference, the caller's arrays are never modified. */
mlem_status mlem_reconstruct(const uint64_t* csr_rows, const uint32_t* csr_cols,
                             const float* csr_vals, const uint64_t* csr_rows_trans,
                             const uint32_t* csr_cols_trans, const float* csr_vals_trans,
                             const int32_t* g, const float* norm, const float* f,
                             float* result_f, uint32_t rows, uint32_t cols, uint64_t nnzs,
                             uint32_t iterations, uint32_t device_numbers,
                             uint32_t matrix_vector_mul, uint32_t secsize_fp,
                             uint32_t secsize_bp, uint32_t using_trans);

/* ----------------------------------------------------- single operators */
/* ratio = correl(g, A·f): forward projection with the fused correlation of
 * calcCorrel (kernel.cu:11-19).  Device pointers, asynchronous on stream.
 * fwproj_out (optional, f32[rows]) receives A·f before the correlation. */
mlem_status mlem_forward_project(mlem_matrix* m, const float* f_dev, const int32_t* g_dev,
                                 float* ratio_dev, float* fwproj_out_dev,
                                 const mlem_run_opts* opts, void* stream);
/* bp = Aᵀ·ratio (no update) into bp_dev f32[cols]. */
mlem_status mlem_back_project(mlem_matrix* m, const float* ratio_dev, float* bp_dev,
                              const mlem_run_opts* opts, void* stream);

/* Merge-path partition search of merge_based_start (kernel.cu:190-241) for
 * the thread starts d = t*secsize, t = 0..nthreads-1, over device row
 * pointers u64[rows+1].  Writes the coordinates (i, j) as int64. */
mlem_status mlem_merge_path_search(const uint64_t* rowptr_dev, uint32_t rows, uint64_t nnz,
                                   uint32_t secsize, uint64_t nthreads, int64_t* i_out_dev,
                                   int64_t* j_out_dev, void* stream);

/* Merge-path forward projection with the fused correlation, like
 * mlem_forward_project with MLEM_SPMV_MERGE, for callers that must not
 * allocate device memory (an allocation during graph capture or inside a
 * host-owned memory pool is not possible for them).  No counterpart in the
 * reference.  It allocates nothing: its per-tile scratch is a fixed 4 MiB
 * device array inside the library, held by every GPU that loads the library
 * until exit, which limits rows + nnz to about 220 million at secsize 5
 * (larger inputs return MLEM_EINVAL with the limit in the message).  The
 * first call on a device looks the array up (cudaGetSymbolAddress), and again
 * after the device's context was re-created (cudaDeviceReset); make that first
 * call before any stream capture.  All calls share the array: calls that
 * overlap on the GPU race, so serialise them.  Device pointers in, ratio
 * f32[rows] out; nnz must equal rowptr_dev[rows] and col[e] < cols; secsize
 * 1..125; asynchronous on `stream`. */
mlem_status mlem_forward_project_merge_noalloc(const uint64_t* rowptr_dev, const uint32_t* col_dev,
                                               const float* val_dev, uint32_t rows, uint32_t cols,
                                               uint64_t nnz, const float* x_dev, const int32_t* g_dev,
                                               float* ratio_dev, uint32_t secsize, void* stream);

/* GPU stable counting-sort transpose (CSR -> CSR of Aᵀ), bit-exact with
 * sptrans_scanTrans_specialized (sptrans.h:397-545).  Host in/out buffers. */
mlem_status mlem_transpose_host(const mlem_csr_host* csr, uint64_t* colptr, uint32_t* rowidx,
                                float* val);

/* Column sums Aᵀ1 accumulated in FP64 on the GPU, rounded to f32 (replaces
 * calcColumnSums, main.cu:558-580).  Host in/out buffers. */
mlem_status mlem_column_sums_host(const mlem_csr_host* csr, float* norm_out);

/* nnz-balanced row partition of partitionMatrix (main.cu:593-611): segments
 * u32[nseg+1], seg_rows u32[nseg], seg_nnz u32[nseg], offsets u64[nseg]. */
mlem_status mlem_partition_rows(const uint64_t* rowptr, uint64_t nnz, uint32_t rows,
                                uint32_t nseg, uint32_t* segments, uint32_t* seg_rows,
                                uint32_t* seg_nnz, uint64_t* offsets);

/* ------------------------------------------------------------- file I/O */
typedef struct {
    uint32_t rows, cols;
    uint64_t nnz;
    uint8_t sym_flags;          /* csr4 header byte 5 (x/y/z symmetry bits) */
    uint32_t nx, ny, nz;        /* voxel grid from the scanner configuration */
} mlem_csr4_header;

/* Parses only the header and scanner configuration of a csr4 file. */
mlem_status mlem_csr4_read_header(const char* path, mlem_csr4_header* hdr);
/* Reads a whole csr4 file into caller buffers: rowptr u64[rows+1] (with a
 * leading 0, like csr_format_for_cuda), col u32[nnz], val f32[nnz]. */
mlem_status mlem_csr4_read(const char* path, uint64_t* rowptr, uint32_t* col, float* val);

/* Scanner description written into a csr4 header. */
typedef struct {
    uint32_t n_layers;          /* layers written with {w,h,d,r,mu} below */
    float crystal_w, crystal_h, crystal_d, radius, mu;
    uint32_t n_blocks, block_size, n_rings;
    float block_gap, ring_gap;
    float voxel_w, voxel_h, voxel_d;
    uint32_t nx, ny, nz;
    uint8_t sym_flags;
} mlem_csr4_scanner;

/* Writes a csr4 file readable by the reference Csr4Matrix. */
mlem_status mlem_csr4_write(const char* path, const mlem_csr4_scanner* scanner,
                            const mlem_csr_host* csr);
/* Raw headerless vectors (vector.hpp:33-87): int32 sinogram in, f32 image out. */
mlem_status mlem_read_sinogram(const char* path, int32_t* g, uint64_t capacity,
                               uint64_t* count_out);
mlem_status mlem_write_image(const char* path, const float* f, uint64_t count);

/* ------------------------------------------------ synthetic system matrix */
/* Cylindrical ring scanner: n_rings rings of det_per_ring detectors on a
 * circle of `radius` mm, ring centres at z = (k - (n_rings-1)/2)*ring_pitch;
 * voxel grid nx*ny*nz of (vx,vy,vz) mm centred on the origin.  Rows are the
 * unordered detector pairs (a<b) in lexicographic order, columns
 * x + nx*(y + ny*z), values the exact Siddon ray-voxel intersection lengths
 * in mm (averaged over the sub-rays of the tube of response), columns
 * strictly ascending within a row. */
typedef struct {
    uint32_t det_per_ring, n_rings;
    float radius, ring_pitch;
    uint32_t nx, ny, nz;
    float vx, vy, vz;
    uint32_t row_stride;        /* 0 or 1: all rows; k > 1: keep rows r with r % k == row_phase */
    uint32_t row_phase;
    /* Tube of response: sub_t x sub_z parallel sub-rays per LOR spread over
     * width_t (tangential) x width_z (axial) mm of the crystal faces; the
     * element value is the mean intersection length over the sub-rays.
     * 0 or 1 sub-rays = the single line between the crystal centres. */
    uint32_t sub_t, sub_z;
    float width_t, width_z;
} mlem_geometry;

/* Number of rows (kept LORs) of the geometry; 0 for an invalid geometry. */
uint64_t mlem_siddon_rows(const mlem_geometry* geo);
/* Row pointers u64[rows+1] of the geometry's matrix (host, OpenMP). */
mlem_status mlem_siddon_count_host(const mlem_geometry* geo, uint64_t* rowptr_out);
/* Fills col/val for rows with the given rowptr (host, OpenMP). */
mlem_status mlem_siddon_fill_host(const mlem_geometry* geo, const uint64_t* rowptr,
                                  uint32_t* col, float* val);
/* Same generator on the GPU: the matrix is built in HBM and never leaves it.
 * Bit-identical to the host generator (no FMA contraction, same operation order). */
mlem_status mlem_matrix_generate(const mlem_geometry* geo, const mlem_matrix_opts* opts,
                                 mlem_matrix** out);
/* Copies the device matrix A to host buffers (f32 values converted back). */
mlem_status mlem_matrix_get_csr(const mlem_matrix* m, uint64_t* rowptr, uint32_t* col,
                                float* val);

/* ------------------------------------------------------------- batched */
/* Reconstructs `count` sinograms against one resident matrix as a batched
 * SpMM (forward and back projection shared by up to 32 instances per tile),
 * replayed as CUDA graphs.  The tile's slots are a pool: an instance that has
 * run its iterations hands its image back and the next instance takes its slot
 * before the following iteration.  g: i32[count][rows]; iterations: u32[count]
 * (uneven counts allowed, 0 returns the initial image); f0: NULL (reference
 * initial value per instance) or f32[count][cols]; f_out: f32[count][cols].
 * An instance's image is bit-identical whichever tile, slot and company it
 * runs in. */
typedef struct {
    uint32_t tile;              /* instances per batch tile: 0 = autotune, else 8/16/32 */
    uint32_t use_graph;
    uint32_t order_by_iterations; /* 1: instances enter the pool longest first */
    uint32_t form;              /* 0 = autotuned per matrix; 1 = one CUDA graph per iteration (forward
                                   and back projection launches); 2 = persistent: the iterations
                                   between two slot refills run in one cooperative launch, forward
                                   and back projection separated by grid-wide barriers (needs Aᵀ;
                                   a barrier wait that runs out returns MLEM_ETIMEOUT).  Every form
                                   gives the same bits. */
} mlem_batch_opts;

void mlem_batch_opts_default(mlem_batch_opts* o);
mlem_status mlem_batch_run(mlem_matrix* m, uint32_t count, const int32_t* g,
                           const uint32_t* iterations, const float* f0,
                           const mlem_batch_opts* opts, float* f_out, mlem_stats* stats);

/* -------------------------------------------------------------- serving */
typedef struct mlem_server mlem_server;

typedef struct {
    uint32_t slots_per_matrix;  /* concurrent reconstructions per matrix (batch tile 8/16/32,
                                   0 = the tile the batch autotuner picks for each matrix) */
    uint64_t hbm_budget_bytes;  /* admission limit for per-request state (0 = free HBM - reserve) */
    uint64_t hbm_reserve_bytes; /* HBM kept free when hbm_budget_bytes == 0 */
    uint32_t queue_capacity;    /* max queued requests before submit returns EBUSY */
    uint32_t stream_priority;   /* per-matrix stream priority: 0 = by size (< 16 M nonzeros
                                   highest, < 512 M middle, larger lowest), 1 (default) = small
                                   matrices (< 16 M nonzeros) highest, all others equal,
                                   2 = all equal */
} mlem_server_opts;

void mlem_server_opts_default(mlem_server_opts* o);
mlem_status mlem_server_create(const mlem_server_opts* opts, mlem_server** out);
/* Registers a resident matrix; returns its index in *matrix_id.  The server
 * does not take ownership: destroy the matrix after the server. */
mlem_status mlem_server_add_matrix(mlem_server* s, mlem_matrix* m, uint32_t* matrix_id);
/* Queues a reconstruction; g (i32[rows]) is copied at submit time.
 * *request_id identifies it for mlem_server_wait. */
mlem_status mlem_server_submit(mlem_server* s, uint32_t matrix_id, const int32_t* g,
                               uint32_t iterations, uint64_t* request_id);
/* Waits up to timeout_ms for a request; copies its image to f_out
 * (f32[cols]) and its submit->done latency in seconds. */
mlem_status mlem_server_wait(mlem_server* s, uint64_t request_id, float* f_out,
                             uint32_t timeout_ms, double* latency_s);
/* Cancels a queued request (MLEM_EINVAL if unknown or already running). */
mlem_status mlem_server_cancel(mlem_server* s, uint64_t request_id);
typedef struct {
    uint64_t submitted, completed, cancelled, rejected;
    uint64_t active, queued;
    uint64_t hbm_in_use;
    uint64_t iterations_done;
} mlem_server_stats;
mlem_status mlem_server_get_stats(mlem_server* s, mlem_server_stats* st);
mlem_status mlem_server_destroy(mlem_server* s);

/* ---------------------------------------------------------- diagnostics */
/* Number of kernels this library launched since load (all entry points). */
uint64_t mlem_kernel_launch_count(void);

#ifdef __cplusplus
}
#endif
#endif /* MLEM_GB300_H */
