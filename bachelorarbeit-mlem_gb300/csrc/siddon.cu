// siddon.cu — synthetic PET system matrix: exact ray/voxel intersection
// lengths (Siddon 1985, incremental traversal with the voxel of each segment
// taken at the segment midpoint) for every unordered detector pair of a
// cylindrical ring scanner.
//
// The same __host__ __device__ ray routine runs on the host (OpenMP) and on
// the GPU.  This translation unit is compiled without FMA contraction on both
// sides (-fmad=false, -ffp-contract=off) and the ray code uses only IEEE
// +,-,*,/, sqrt, floor and ceil, so both generators produce bit-identical
// matrices.  Columns follow scannerconfig.cpp:30-35 (x + nx*(y + ny*z)) and
// are sorted ascending within a row.
#include "kernels.cuh"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

namespace mlem {

namespace {

struct Geo {
    uint32_t dpr, rings, D;      // detectors per ring, rings, total detectors
    double radius, pitch;
    uint32_t nx, ny, nz;
    double vx, vy, vz;
    double x0, y0, z0;           // grid min corner
    uint64_t nlor;               // D*(D-1)/2
    uint64_t stride, phase;
    uint64_t nrows;              // rows kept
    uint32_t sub_t, sub_z, S;    // sub-rays of the tube of response
    double width_t, width_z;
    uint32_t cap_ray;            // max elements of one sub-ray
};

constexpr double kMinLen = 1e-6;  // mm; shorter clips are dropped
constexpr int kMaxDet = 16384;

Geo make_geo(const mlem_geometry& g) {
    Geo G;
    G.dpr = g.det_per_ring;
    G.rings = g.n_rings;
    G.D = g.det_per_ring * g.n_rings;
    G.radius = g.radius;
    G.pitch = g.ring_pitch;
    G.nx = g.nx; G.ny = g.ny; G.nz = g.nz;
    G.vx = g.vx; G.vy = g.vy; G.vz = g.vz;
    G.x0 = -0.5 * G.nx * G.vx;
    G.y0 = -0.5 * G.ny * G.vy;
    G.z0 = -0.5 * G.nz * G.vz;
    G.nlor = (uint64_t)G.D * (G.D - 1) / 2;
    G.stride = g.row_stride > 1 ? g.row_stride : 1;
    G.phase = g.row_stride > 1 ? g.row_phase : 0;
    G.nrows = G.nlor > G.phase ? (G.nlor - G.phase + G.stride - 1) / G.stride : 0;
    G.sub_t = g.sub_t > 1 ? g.sub_t : 1;
    G.sub_z = g.sub_z > 1 ? g.sub_z : 1;
    G.S = G.sub_t * G.sub_z;
    G.width_t = g.width_t;
    G.width_z = g.width_z;
    // a straight segment visits at most nx+ny+nz+4 voxels (one per plane
    // crossed); ray_walk never emits more than cap_ray elements
    G.cap_ray = g.nx + g.ny + g.nz + 8;
    return G;
}

void check_geo(const mlem_geometry& g) {
    MLEM_REQUIRE(g.det_per_ring >= 1 && g.n_rings >= 1, MLEM_EINVAL, "geometry: no detectors");
    MLEM_REQUIRE((uint64_t)g.det_per_ring * g.n_rings >= 2 &&
                     (uint64_t)g.det_per_ring * g.n_rings <= kMaxDet,
                 MLEM_EINVAL, "geometry: detector count out of range");
    MLEM_REQUIRE(g.nx >= 1 && g.ny >= 1 && g.nz >= 1, MLEM_EINVAL, "geometry: empty voxel grid");
    MLEM_REQUIRE((uint64_t)g.nx * g.ny * g.nz < (1ull << 32), MLEM_EUNSUPPORTED, "geometry: too many voxels");
    MLEM_REQUIRE(g.vx > 0 && g.vy > 0 && g.vz > 0 && g.radius > 0, MLEM_EINVAL,
                 "geometry: voxel size and radius must be positive");
    MLEM_REQUIRE(g.row_stride <= 1 || g.row_phase < g.row_stride, MLEM_EINVAL,
                 "geometry: row_phase must be < row_stride");
    const uint32_t st = g.sub_t > 1 ? g.sub_t : 1, sz = g.sub_z > 1 ? g.sub_z : 1;
    MLEM_REQUIRE(st * sz <= 32, MLEM_EINVAL, "geometry: at most 32 sub-rays per LOR");
    MLEM_REQUIRE(g.width_t >= 0 && g.width_z >= 0, MLEM_EINVAL, "geometry: negative tube width");
}

__host__ __device__ __forceinline__ uint64_t lor_start(uint64_t a, uint64_t D) {
    return a * D - a * (a + 1) / 2;
}

// LOR index -> detector pair (a < b), lexicographic order.
__host__ __device__ __forceinline__ void lor_pair(uint64_t r, uint64_t D, uint32_t& a, uint32_t& b) {
    uint64_t lo = 0, hi = D - 2;
    while (lo < hi) {
        const uint64_t mid = (lo + hi + 1) >> 1;
        if (lor_start(mid, D) <= r) lo = mid;
        else hi = mid - 1;
    }
    a = (uint32_t)lo;
    b = (uint32_t)(r - lor_start(lo, D) + lo + 1);
}

__host__ __device__ __forceinline__ void det_pos(const Geo& G, const double* ct, const double* st,
                                                 uint32_t d, double& x, double& y, double& z) {
    const uint32_t ring = d / G.dpr, k = d % G.dpr;
    x = G.radius * ct[k];
    y = G.radius * st[k];
    z = ((double)ring - 0.5 * (double)(G.rings - 1)) * G.pitch;
}

struct AxisWalk {
    double next;   // alpha of the next plane crossing (+inf if none)
    int64_t plane; // index of that plane
    int dir;       // +1 / -1 / 0
};

__host__ __device__ __forceinline__ bool axis_range(double p1, double d, double lo, int n, double v,
                                                    double& amin, double& amax) {
    const double hi = lo + (double)n * v;
    if (d != 0.0) {
        const double a0 = (lo - p1) / d, an = (hi - p1) / d;
        amin = fmax(amin, fmin(a0, an));
        amax = fmin(amax, fmax(a0, an));
        return true;
    }
    return p1 > lo && p1 < hi;  // parallel ray must lie strictly inside the slab
}

__host__ __device__ __forceinline__ AxisWalk axis_start(double p1, double d, double lo, double v,
                                                        double amin) {
    AxisWalk w;
    if (d > 0.0) {
        w.dir = 1;
        w.plane = (int64_t)floor((p1 + amin * d - lo) / v) + 1;
        w.next = (lo + (double)w.plane * v - p1) / d;
    } else if (d < 0.0) {
        w.dir = -1;
        w.plane = (int64_t)ceil((p1 + amin * d - lo) / v) - 1;
        w.next = (lo + (double)w.plane * v - p1) / d;
    } else {
        w.dir = 0;
        w.plane = 0;
        w.next = 1e300;
    }
    return w;
}

__host__ __device__ __forceinline__ void axis_advance(AxisWalk& w, double p1, double d, double lo,
                                                      double v) {
    w.plane += w.dir;
    w.next = (lo + (double)w.plane * v - p1) / d;
}

__host__ __device__ __forceinline__ int64_t clampi(int64_t v, int64_t n) {
    return v < 0 ? 0 : (v >= n ? n - 1 : v);
}

// End points of sub-ray k of LOR (a, b): offsets u (tangential) and v
// (axial) across the crystal faces, mirrored at b so that the sub-rays of
// facing detectors are parallel.
__host__ __device__ __forceinline__ void sub_ray(const Geo& G, const double* ct, const double* st,
                                                 uint32_t a, uint32_t b, uint32_t k, double p[6]) {
    const uint32_t i = k % G.sub_t, j = k / G.sub_t;
    const double u = ((double)i + 0.5) / (double)G.sub_t - 0.5;
    const double v = (((double)j + 0.5) / (double)G.sub_z - 0.5) * G.width_z;
    const double ut = u * G.width_t;
    const uint32_t ka = a % G.dpr, kb = b % G.dpr;
    det_pos(G, ct, st, a, p[0], p[1], p[2]);
    det_pos(G, ct, st, b, p[3], p[4], p[5]);
    p[0] = p[0] - ut * st[ka];
    p[1] = p[1] + ut * ct[ka];
    p[2] = p[2] + v;
    p[3] = p[3] + ut * st[kb];
    p[4] = p[4] - ut * ct[kb];
    p[5] = p[5] + v;
}

// Walks the segment p[0..2] -> p[3..5] through the grid and calls
// emit(col, len) once per intersected voxel (len in mm, double).
template <class Emit>
__host__ __device__ uint32_t ray_walk(const Geo& G, const double p[6], Emit&& emit) {
    const double p1x = p[0], p1y = p[1], p1z = p[2], p2x = p[3], p2y = p[4], p2z = p[5];
    const double dx = p2x - p1x, dy = p2y - p1y, dz = p2z - p1z;
    const double L = sqrt(dx * dx + dy * dy + dz * dz);
    double amin = 0.0, amax = 1.0;
    if (!axis_range(p1x, dx, G.x0, G.nx, G.vx, amin, amax)) return 0;
    if (!axis_range(p1y, dy, G.y0, G.ny, G.vy, amin, amax)) return 0;
    if (!axis_range(p1z, dz, G.z0, G.nz, G.vz, amin, amax)) return 0;
    if (!(amax > amin)) return 0;
    AxisWalk wx = axis_start(p1x, dx, G.x0, G.vx, amin);
    AxisWalk wy = axis_start(p1y, dy, G.y0, G.vy, amin);
    AxisWalk wz = axis_start(p1z, dz, G.z0, G.vz, amin);
    double acur = amin;
    uint32_t n = 0;
    // consecutive segments that land in the same voxel (a plane crossing
    // absorbed by rounding) are merged into one element
    uint32_t pend_col = 0xffffffffu;
    double pend_len = 0.0;
    auto flush = [&]() {
        if (pend_col != 0xffffffffu && pend_len > kMinLen && n < G.cap_ray) {
            emit(pend_col, pend_len);
            ++n;
        }
    };
    const uint32_t guard = G.nx + G.ny + G.nz + 8;
    for (uint32_t it = 0; it < 2 * guard && acur < amax; ++it) {
        const double an = fmin(fmin(wx.next, wy.next), fmin(wz.next, amax));
        if (an > acur) {
            const double am = 0.5 * (acur + an);
            const int64_t ix = clampi((int64_t)floor((p1x + am * dx - G.x0) / G.vx), G.nx);
            const int64_t iy = clampi((int64_t)floor((p1y + am * dy - G.y0) / G.vy), G.ny);
            const int64_t iz = clampi((int64_t)floor((p1z + am * dz - G.z0) / G.vz), G.nz);
            const uint32_t c = (uint32_t)(ix + (int64_t)G.nx * (iy + (int64_t)G.ny * iz));
            const double len = (an - acur) * L;
            if (c == pend_col) {
                pend_len += len;
            } else {
                flush();
                pend_col = c;
                pend_len = len;
            }
        }
        acur = an;
        if (wx.dir && wx.next <= an) axis_advance(wx, p1x, dx, G.x0, G.vx);
        if (wy.dir && wy.next <= an) axis_advance(wy, p1y, dy, G.y0, G.vy);
        if (wz.dir && wz.next <= an) axis_advance(wz, p1z, dz, G.z0, G.vz);
    }
    flush();
    return n;
}

// Sort key of a sub-ray element: column, then sub-ray index.
__host__ __device__ __forceinline__ uint64_t sub_key(uint32_t c, uint32_t k) {
    return ((uint64_t)c << 5) | k;
}

struct HostEntry {
    uint64_t key;
    double len;
};

// Union of the sub-rays of row q (host): elements sorted by (column, sub-ray),
// equal columns summed in sub-ray order, value = sum / S.  Calls
// out(col, value) in ascending column order; returns the element count.
template <class Out>
uint32_t row_host(const Geo& G, const double* ct, const double* st, uint64_t q,
                  std::vector<HostEntry>& buf, Out&& out) {
    uint32_t a, b;
    lor_pair(q * G.stride + G.phase, G.D, a, b);
    buf.clear();
    for (uint32_t k = 0; k < G.S; ++k) {
        double p[6];
        sub_ray(G, ct, st, a, b, k, p);
        ray_walk(G, p, [&](uint32_t c, double len) { buf.push_back({sub_key(c, k), len}); });
    }
    std::sort(buf.begin(), buf.end(), [](const HostEntry& x, const HostEntry& y) { return x.key < y.key; });
    uint32_t n = 0;
    for (size_t i = 0; i < buf.size();) {
        const uint64_t c = buf[i].key >> 5;
        double sum = 0.0;
        size_t j = i;
        for (; j < buf.size() && (buf[j].key >> 5) == c; ++j) sum += buf[j].len;
        out((uint32_t)c, (float)(sum / (double)G.S));
        ++n;
        i = j;
    }
    return n;
}

// One warp per row (device): lane k < S traces sub-ray k into its slice of
// the warp's shared buffer, the warp sorts (key, len) bitonically, then
// element starts are found with a ballot and each start sums its run in
// sub-ray order.  FILL = false writes counts, true writes the row.
template <bool FILL>
__global__ void k_sid_rows(Geo G, const double* __restrict__ ct, const double* __restrict__ st,
                           uint32_t mcap, uint32_t* __restrict__ cnt, const uint64_t* __restrict__ rowptr,
                           uint32_t* __restrict__ col, float* __restrict__ val) {
    extern __shared__ __align__(16) unsigned char sm[];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    uint64_t* key = reinterpret_cast<uint64_t*>(sm) + (size_t)w * mcap * 2;
    double* len = reinterpret_cast<double*>(key + mcap);
    const uint64_t nw = (gridDim.x * (uint64_t)blockDim.x) >> 5;
    for (uint64_t q = (blockIdx.x * (uint64_t)blockDim.x + threadIdx.x) >> 5; q < G.nrows; q += nw) {
        for (uint32_t i = lane; i < mcap; i += 32) key[i] = ~0ull;
        __syncwarp();
        uint32_t a, b;
        lor_pair(q * G.stride + G.phase, G.D, a, b);
        if ((uint32_t)lane < G.S) {
            double p[6];
            sub_ray(G, ct, st, a, b, (uint32_t)lane, p);
            uint32_t pos = (uint32_t)lane * G.cap_ray;
            ray_walk(G, p, [&](uint32_t c, double l) {
                key[pos] = sub_key(c, (uint32_t)lane);
                len[pos] = l;
                ++pos;
            });
        }
        __syncwarp();
        for (uint32_t k = 2; k <= mcap; k <<= 1) {
            for (uint32_t j = k >> 1; j > 0; j >>= 1) {
                for (uint32_t i = lane; i < mcap; i += 32) {
                    const uint32_t p = i ^ j;
                    if (p > i) {
                        const bool up = (i & k) == 0;
                        if ((key[i] > key[p]) == up) {
                            const uint64_t tk = key[i]; key[i] = key[p]; key[p] = tk;
                            const double tl = len[i]; len[i] = len[p]; len[p] = tl;
                        }
                    }
                }
                __syncwarp();
            }
        }
        uint32_t base = 0;
        const uint64_t out0 = FILL ? rowptr[q] : 0;
        for (uint32_t i0 = 0; i0 < mcap; i0 += 32) {
            const uint32_t i = i0 + lane;
            const uint64_t kk = key[i];
            const bool valid = kk != ~0ull;
            const bool start = valid && (i == 0 || (key[i - 1] >> 5) != (kk >> 5));
            const unsigned bal = __ballot_sync(0xffffffffu, start);
            if (FILL && start) {
                double sum = 0.0;
                for (uint32_t j = i; j < mcap && key[j] != ~0ull && (key[j] >> 5) == (kk >> 5); ++j) sum += len[j];
                const uint64_t o = out0 + base + __popc(bal & ((1u << lane) - 1u));
                col[o] = (uint32_t)(kk >> 5);
                val[o] = (float)(sum / (double)G.S);
            }
            base += __popc(bal);
            if (__ballot_sync(0xffffffffu, valid) != 0xffffffffu) break;
        }
        if (!FILL && lane == 0) cnt[q] = base;
        __syncwarp();
    }
}

uint32_t pow2_at_least(uint32_t n) {
    uint32_t m = 32;
    while (m < n) m <<= 1;
    return m;
}

void angle_tables(const Geo& G, std::vector<double>& ct, std::vector<double>& st) {
    ct.resize(G.dpr);
    st.resize(G.dpr);
    const double two_pi = 6.283185307179586476925286766559;
    for (uint32_t k = 0; k < G.dpr; ++k) {
        const double th = two_pi * (double)k / (double)G.dpr;
        ct[k] = std::cos(th);
        st[k] = std::sin(th);
        // exact zeros on the axes, so rays along a grid plane are parallel to it
        if (std::fabs(ct[k]) < 1e-12) ct[k] = 0.0;
        if (std::fabs(st[k]) < 1e-12) st[k] = 0.0;
    }
}

}  // namespace

uint64_t siddon_rows(const mlem_geometry& g) {
    check_geo(g);
    return make_geo(g).nrows;
}

void siddon_count_host(const mlem_geometry& g, uint64_t* rowptr) {
    check_geo(g);
    const Geo G = make_geo(g);
    std::vector<double> ct, st;
    angle_tables(G, ct, st);
    rowptr[0] = 0;
#pragma omp parallel
    {
        std::vector<HostEntry> buf;
#pragma omp for schedule(dynamic, 256)
        for (int64_t q = 0; q < (int64_t)G.nrows; ++q)
            rowptr[q + 1] = row_host(G, ct.data(), st.data(), (uint64_t)q, buf, [](uint32_t, float) {});
    }
    for (uint64_t q = 0; q < G.nrows; ++q) rowptr[q + 1] += rowptr[q];
}

void siddon_fill_host(const mlem_geometry& g, const uint64_t* rowptr, uint32_t* col, float* val) {
    check_geo(g);
    const Geo G = make_geo(g);
    std::vector<double> ct, st;
    angle_tables(G, ct, st);
#pragma omp parallel
    {
        std::vector<HostEntry> buf;
#pragma omp for schedule(dynamic, 256)
        for (int64_t q = 0; q < (int64_t)G.nrows; ++q) {
            uint64_t pos = rowptr[q];
            row_host(G, ct.data(), st.data(), (uint64_t)q, buf, [&](uint32_t c, float v) {
                col[pos] = c;
                val[pos] = v;
                ++pos;
            });
        }
    }
}

void siddon_rows_of_lors(const mlem_geometry& g, const std::vector<uint64_t>& lors, std::vector<uint64_t>& rowptr,
                         std::vector<uint32_t>& col, std::vector<float>& val) {
    check_geo(g);
    Geo G = make_geo(g);
    MLEM_REQUIRE(G.stride == 1, MLEM_EINVAL, "rows of a LOR list need row_stride 1");
    std::vector<double> ct, st;
    angle_tables(G, ct, st);
    const int64_t n = (int64_t)lors.size();
    rowptr.assign(lors.size() + 1, 0);
#pragma omp parallel
    {
        std::vector<HostEntry> buf;
#pragma omp for schedule(dynamic, 256)
        for (int64_t q = 0; q < n; ++q)
            rowptr[q + 1] = row_host(G, ct.data(), st.data(), lors[q], buf, [](uint32_t, float) {});
    }
    for (int64_t q = 0; q < n; ++q) rowptr[q + 1] += rowptr[q];
    col.resize(rowptr[n]);
    val.resize(rowptr[n]);
#pragma omp parallel
    {
        std::vector<HostEntry> buf;
#pragma omp for schedule(dynamic, 256)
        for (int64_t q = 0; q < n; ++q) {
            uint64_t pos = rowptr[q];
            row_host(G, ct.data(), st.data(), lors[q], buf, [&](uint32_t c, float v) {
                col[pos] = c;
                val[pos] = v;
                ++pos;
            });
        }
    }
}

std::vector<uint32_t> siddon_lor_order(const mlem_geometry& g) {
    check_geo(g);
    const Geo G = make_geo(g);
    std::vector<uint32_t> ord;
    if (G.stride != 1) return ord;  // sampled matrices keep their order
    ord.reserve(G.nrows);
    const uint32_t T = 4;
    for (uint32_t ra = 0; ra < G.rings; ++ra)
        for (uint32_t rb = ra; rb < G.rings; ++rb)
            for (uint32_t i = 0; i < G.dpr; i += T)
                for (uint32_t j = 0; j < G.dpr; j += T)
                    for (uint32_t ka = i; ka < std::min(i + T, G.dpr); ++ka)
                        for (uint32_t kb = j; kb < std::min(j + T, G.dpr); ++kb) {
                            const uint64_t a = (uint64_t)ra * G.dpr + ka, b = (uint64_t)rb * G.dpr + kb;
                            if (a < b) ord.push_back((uint32_t)(lor_start(a, G.D) + (b - a - 1)));
                        }
    return ord;
}

std::vector<uint32_t> voxel_brick_order(uint32_t nx, uint32_t ny, uint32_t nz, uint32_t bx, uint32_t by,
                                        uint32_t bz) {
    std::vector<uint32_t> ord;
    ord.reserve((uint64_t)nx * ny * nz);
    for (uint32_t z0 = 0; z0 < nz; z0 += bz)
        for (uint32_t y0 = 0; y0 < ny; y0 += by)
            for (uint32_t x0 = 0; x0 < nx; x0 += bx)
                for (uint32_t z = z0; z < std::min(z0 + bz, nz); ++z)
                    for (uint32_t y = y0; y < std::min(y0 + by, ny); ++y)
                        for (uint32_t x = x0; x < std::min(x0 + bx, nx); ++x)
                            ord.push_back(x + nx * (y + ny * z));
    return ord;
}

void siddon_generate_device(const mlem_geometry& g, DevCsr& A, cudaStream_t s) {
    check_geo(g);
    const Geo G = make_geo(g);
    MLEM_REQUIRE(G.nrows < (1ull << 32), MLEM_EUNSUPPORTED, "geometry: too many rows");
    const uint32_t mcap = pow2_at_least(G.S * G.cap_ray);
    const size_t per_warp = (size_t)mcap * 16;
    MLEM_REQUIRE(per_warp <= 200 * 1024, MLEM_EUNSUPPORTED,
                 "geometry: sub-rays x grid too large for the device generator");
    const int warps = (int)std::max<size_t>(1, std::min<size_t>(4, (96 * 1024) / per_warp));
    const size_t smem = per_warp * warps;
    std::vector<double> ct, st;
    angle_tables(G, ct, st);
    double* dtab = nullptr;
    MLEM_CUDA(cudaMallocAsync(&dtab, sizeof(double) * 2 * G.dpr, s));
    MLEM_CUDA(cudaMemcpyAsync(dtab, ct.data(), sizeof(double) * G.dpr, cudaMemcpyHostToDevice, s));
    MLEM_CUDA(cudaMemcpyAsync(dtab + G.dpr, st.data(), sizeof(double) * G.dpr, cudaMemcpyHostToDevice, s));
    A.nrows = (uint32_t)G.nrows;
    A.ncols = G.nx * G.ny * G.nz;
    A.vt = MLEM_VAL_F32;
    uint32_t* cnt = nullptr;
    MLEM_CUDA(cudaMallocAsync(&cnt, sizeof(uint32_t) * std::max<uint64_t>(G.nrows, 1), s));
    MLEM_CUDA(cudaMalloc(&A.rowptr, sizeof(uint64_t) * (G.nrows + 1)));
    MLEM_CUDA(cudaFuncSetAttribute(k_sid_rows<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    MLEM_CUDA(cudaFuncSetAttribute(k_sid_rows<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    const unsigned grid = std::max(1u, std::min<unsigned>(ceil_div_u(G.nrows, warps), 152u * 64u));
    if (G.nrows) {
        k_sid_rows<false><<<grid, warps * 32, smem, s>>>(G, dtab, dtab + G.dpr, mcap, cnt, nullptr, nullptr, nullptr);
        MLEM_LAUNCHED();
    }
    scan_counts_u64(cnt, A.rowptr, G.nrows, s);
    MLEM_CUDA(cudaFreeAsync(cnt, s));
    uint64_t nnz = 0;
    MLEM_CUDA(cudaMemcpyAsync(&nnz, A.rowptr + G.nrows, sizeof(uint64_t), cudaMemcpyDeviceToHost, s));
    MLEM_CUDA(cudaStreamSynchronize(s));
    A.nnz = nnz;
    MLEM_CUDA(cudaMalloc(&A.idx, sizeof(uint32_t) * padded(nnz)));
    MLEM_CUDA(cudaMalloc(&A.val, sizeof(float) * padded(nnz)));
    MLEM_CUDA(cudaMemsetAsync(A.idx, 0, sizeof(uint32_t) * padded(nnz), s));
    MLEM_CUDA(cudaMemsetAsync(A.val, 0, sizeof(float) * padded(nnz), s));
    if (G.nrows) {
        k_sid_rows<true><<<grid, warps * 32, smem, s>>>(G, dtab, dtab + G.dpr, mcap, nullptr, A.rowptr, A.idx,
                                                        (float*)A.val);
        MLEM_LAUNCHED();
    }
    A.max_row = max_row_length(A.rowptr, A.nrows, s);
    MLEM_CUDA(cudaFreeAsync(dtab, s));
    MLEM_CUDA(cudaStreamSynchronize(s));
}

}  // namespace mlem
