// symmetry.cu — symmetry-compressed projections for generated cylindrical
// scanners.
//
// A ring scanner with dpr % 4 == 0 detectors per ring (detector k at angle
// 2*pi*k/dpr), rings placed symmetrically about z = 0 and a square voxel grid
// centred on the axis is invariant under 16 transformations s = q + 4m + 8f:
// a mirror y -> -y (m), a rotation by q * 90 degrees, and the axial flip
// z -> -z (f), applied in that order.  On a voxel (x, y, z) of an n x n x nz
// grid: y -> n-1-y; (x, y) -> (n-1-y, x) q times; z -> nz-1-z.  On a
// detector (ring, k): k -> (dpr-k) % dpr; k -> (k + q*dpr/4) % dpr;
// ring -> rings-1-ring.  A LOR (a, b) maps to the sorted pair of images.
//
// The symmetric matrix A^ is built from the rows of the canonical LORs (the
// smallest index of every orbit), generated as usual and, where a LOR is
// fixed by some transformations, averaged over them so that
// A^[s(r), s(c)] = A^[r, c] holds exactly.  A^ and its transpose stay the
// matrix of the handle (every mode and getter uses them); beside them this
// file keeps two compact operands with 1/16 of the nonzeros each:
//   forward projection: the canonical LOR rows r_k; an entry for voxel
//     c = t(v_j) is stored as j << 4 | t (v_j the canonical voxel of c);
//   back projection over A^T: the canonical voxel rows v_j; an entry for
//     LOR r = t(r_k) is stored as k << 4 | t.
// Row k of the product for transformation s needs the input at s(t(v_j)):
// with the input laid out in orbit order, O[16 j + u] = x[u(v_j)], that is
// O[16 j + (s o t)].  Writing s = F^f R^q M^m (mirror M first, then q
// rotations R, then the axial flip F; M R = R^-1 M, F central),
//   s o t = F^(f_s ^ f_t) R^(q_s + (m_s ? -q_t : q_t)) M^(m_s ^ m_t),
// so for the four s sharing (m_s, f_s) the needed values are one aligned
// float4 of the 64-byte orbit row (chunk (m_s ^ m_t) + 2 (f_s ^ f_t), which
// is (key >> 2) ^ (m_s + 2 f_s) in units of float4), rotated by q_t or -q_t.
// The entries of a row are kept in 4 segments by q_t, so a lane adds the
// float4 unrotated and rotates its sums once per segment.  A warp handles
// one compact row: 8 entries per step, 4 lanes per entry (one per
// (m_s, f_s)), each lane one 16-byte load and 4 sums; the 64 bytes an entry
// needs come in one coalesced piece.  The orbit arrays (16 floats per
// canonical voxel / LOR, L2-resident) are gathered from the natural-order
// input by a small kernel before each projection; each distinct output row
// (LOR s(r_k), voxel s(v_j)) is written by the first s that produces it.
#include "kernels.cuh"

#include <algorithm>
#include <cstring>
#include <functional>
#include <map>
#include <string>
#include <vector>

namespace mlem {

namespace {

struct SymMaps {
    uint32_t n, nz, dpr, rings, D;
    void vox(int s, uint32_t& x, uint32_t& y, uint32_t& z) const {
        if ((s >> 2) & 1) y = n - 1 - y;
        for (int q = 0; q < (s & 3); ++q) {
            const uint32_t t = x;
            x = n - 1 - y;
            y = t;
        }
        if (s >> 3) z = nz - 1 - z;
    }
    uint32_t vox_index(int s, uint32_t c) const {
        uint32_t x = c % n, y = (c / n) % n, z = c / (n * n);
        vox(s, x, y, z);
        return x + n * (y + n * z);
    }
    uint32_t det(int s, uint32_t d) const {
        uint32_t ring = d / dpr, k = d % dpr;
        if ((s >> 2) & 1) k = (dpr - k) % dpr;
        k = (k + (uint32_t)(s & 3) * (dpr / 4)) % dpr;
        if (s >> 3) ring = rings - 1 - ring;
        return ring * dpr + k;
    }
    uint64_t lor(uint64_t a, uint64_t b) const {
        if (a > b) std::swap(a, b);
        return a * D - a * (a + 1) / 2 + (b - a - 1);
    }
};

// comp[s][t]: the transformation "t, then s", found on probe voxels.
void composition(const SymMaps& M, uint8_t comp[16][16], uint8_t inv[16]) {
    SymMaps P = M;
    P.n = 7;
    P.nz = 5;
    const uint32_t probe[3][3] = {{0, 1, 0}, {2, 5, 1}, {3, 0, 4}};
    auto image = [&](int s, const uint32_t p[3], uint32_t out[3]) {
        out[0] = p[0];
        out[1] = p[1];
        out[2] = p[2];
        P.vox(s, out[0], out[1], out[2]);
    };
    for (int s = 0; s < 16; ++s)
        for (int t = 0; t < 16; ++t) {
            int found = -1;
            for (int u = 0; u < 16 && found < 0; ++u) {
                bool same = true;
                for (int k = 0; k < 3 && same; ++k) {
                    uint32_t a[3], b[3], c[3];
                    image(t, probe[k], a);
                    image(s, a, b);
                    image(u, probe[k], c);
                    same = b[0] == c[0] && b[1] == c[1] && b[2] == c[2];
                }
                if (same) found = u;
            }
            MLEM_REQUIRE(found >= 0, MLEM_EINVAL, "internal: symmetry group not closed");
            // the closed form the compact kernels use (k_sym_orbit)
            const int d = ((s >> 2) & 1) ? (4 - (t & 3)) & 3 : (t & 3);
            const int closed = ((s + d) & 3) + 4 * (((s >> 2) ^ (t >> 2)) & 1) + 8 * ((s >> 3) ^ (t >> 3));
            MLEM_REQUIRE(found == closed, MLEM_EINVAL, "internal: symmetry composition differs from its closed form");
            // ... and the detectors (hence LORs) compose the same way as the voxels
            for (uint32_t d = 0; d < M.D; d += std::max(1u, M.D / 61))
                MLEM_REQUIRE(M.det(s, M.det(t, d)) == M.det(closed, d), MLEM_EINVAL,
                             "internal: detector maps compose differently from voxel maps");
            comp[s][t] = (uint8_t)found;
        }
    for (int s = 0; s < 16; ++s)
        for (int t = 0; t < 16; ++t)
            if (comp[s][t] == 0) inv[s] = (uint8_t)t;
}

// ---------------------------------------------------------------- device maps
// s(x, y, z) of a voxel as an index: ax*x + ay*y + az*z + c0 (the map is affine)
struct VoxMap {
    int32_t ax, ay, az, c0;
};

__host__ __device__ __forceinline__ VoxMap vox_map(int s, int32_t n, int32_t nz) {
    auto img = [&](int32_t x, int32_t y, int32_t z) -> int32_t {
        if ((s >> 2) & 1) y = n - 1 - y;
        for (int q = 0; q < (s & 3); ++q) {
            const int32_t t = x;
            x = n - 1 - y;
            y = t;
        }
        if (s >> 3) z = nz - 1 - z;
        return x + n * (y + n * z);
    };
    VoxMap m;
    m.c0 = img(0, 0, 0);
    m.ax = img(1, 0, 0) - m.c0;
    m.ay = img(0, 1, 0) - m.c0;
    m.az = img(0, 0, 1) - m.c0;
    return m;
}

template <typename V>
__device__ __forceinline__ float ld_val(const V* p, uint64_t e) {
    return Val4<V>::one_cached(p, e);
}

// cp.async.bulk.prefetch.L2 of [p, p + bytes) widened to 16-byte granules.
__device__ __forceinline__ void l2_prefetch_range(const void* p, uint64_t bytes) {
    const uint64_t a = reinterpret_cast<uint64_t>(p);
    const uint64_t lo = a & ~15ull, hi = (a + bytes + 15) & ~15ull;
    for (uint64_t q = lo; q < hi; q += 65536) {
        const uint32_t n = (uint32_t)(hi - q < 65536 ? hi - q : 65536);
        asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;" ::"l"(q), "r"(n) : "memory");
    }
}

__device__ __forceinline__ float comp4(const float4& v, int i) {
    return i == 0 ? v.x : (i == 1 ? v.y : (i == 2 ? v.z : v.w));
}

// One step of a segment: UU entries per lane (entries base + slot + 8u),
// predicated when PRED (the last step of a segment).
template <typename V, int UU, bool PRED>
__device__ __forceinline__ void orbit_step(const uint32_t* __restrict__ kp, const V* __restrict__ vp,
                                           const float4* __restrict__ orb, uint32_t base, uint32_t n,
                                           uint32_t slot, uint32_t lb, float4& sa) {
    uint32_t kk[UU];
    float v[UU];
    float4 o[UU];
#pragma unroll
    for (int u = 0; u < UU; ++u) {
        const uint32_t i = base + slot + 8 * u;
        const bool ok = !PRED || i < n;
        kk[u] = ok ? ld_cached(kp + i) : 0u;
        v[u] = ok ? ld_val<V>(vp, i) : 0.f;
    }
#pragma unroll
    for (int u = 0; u < UU; ++u) {
        const bool ok = !PRED || base + slot + 8 * u < n;
        o[u] = ok ? __ldg(orb + ((kk[u] >> 2) ^ lb)) : make_float4(0.f, 0.f, 0.f, 0.f);
    }
#pragma unroll
    for (int u = 0; u < UU; ++u) {
        sa.x = fmaf(v[u], o[u].x, sa.x);
        sa.y = fmaf(v[u], o[u].y, sa.y);
        sa.z = fmaf(v[u], o[u].z, sa.z);
        sa.w = fmaf(v[u], o[u].w, sa.w);
    }
}

// Segment Q of a compact row (entries with q_t = Q): unrotated sums, then
// acc[p] += sums[(p + d) & 3] with d = Q (m_s = 0) or -Q (m_s = 1).
// Warp-uniform steps of 8·U entries, then one predicated step of 8·U'
// entries, U' the smallest power of two that covers the remainder.
template <typename V, int U, int Q>
__device__ __forceinline__ void orbit_segment(const uint32_t* __restrict__ key, const V* __restrict__ val,
                                              const float4* __restrict__ orb, uint64_t s0, uint64_t s1,
                                              uint32_t slot, uint32_t lb, uint32_t mg, float (&acc)[4]) {
    float4 sa = make_float4(0.f, 0.f, 0.f, 0.f);
    // row-local 32-bit offsets
    const uint32_t* kp = key + s0;
    const V* vp = val + s0;
    const uint32_t n = (uint32_t)(s1 - s0);
    uint32_t base = 0;
    for (; base + 8 * U <= n; base += 8 * U) orbit_step<V, U, false>(kp, vp, orb, base, n, slot, lb, sa);
    const uint32_t rem = n - base;  // < 8 U, the same in every lane
    if (rem > 0) {
        if (U >= 8 && rem > 32) orbit_step<V, (U >= 8 ? 8 : 1), true>(kp, vp, orb, base, n, slot, lb, sa);
        else if (U >= 4 && rem > 16) orbit_step<V, (U >= 4 ? 4 : 1), true>(kp, vp, orb, base, n, slot, lb, sa);
        else if (U >= 2 && rem > 8) orbit_step<V, (U >= 2 ? 2 : 1), true>(kp, vp, orb, base, n, slot, lb, sa);
        else orbit_step<V, 1, true>(kp, vp, orb, base, n, slot, lb, sa);
    }
    constexpr int D0 = Q, D1 = (4 - Q) & 3;
#pragma unroll
    for (int p = 0; p < 4; ++p) acc[p] += mg ? comp4(sa, (p + D1) & 3) : comp4(sa, (p + D0) & 3);
}

// Compact product with epilogue: out row oimg[16 row + s] for every s that
// is its own leader in olead[row] (4 bits per s: the first transformation
// with the same output row).  EPI Correl / Raw (forward projection: rows are
// canonical LORs) or Update / Raw (back projection: canonical voxels).
// Segment q of a row holds the entries with q_t = q; lane l of an entry
// loads chunk (key >> 2) ^ (l & 3) of the orbit row (key >> 4).  U entries
// per lane in flight.
// Blocks of 2 warps (rows differ in length; a small block frees its slot
// early).  Register budget per unroll: U = 2 or 4 -> 24 blocks per SM
// (40 registers), 8 -> 20 (48).
constexpr int kOrbitBlock = 64;
constexpr int orbit_min_blocks(int U) { return U <= 4 ? 24 : 20; }

template <typename V, int EPI, int U>
__global__ void __launch_bounds__(kOrbitBlock, orbit_min_blocks(U))
k_sym_orbit(const uint64_t* __restrict__ rowptr4, const uint32_t* __restrict__ key, const V* __restrict__ val,
            uint32_t nrows, const float4* __restrict__ orb, const uint32_t* __restrict__ oimg,
            const uint64_t* __restrict__ olead,
            const int32_t* __restrict__ g, float* __restrict__ out,
            float* __restrict__ fwproj, float* __restrict__ f, const float* __restrict__ norm,
            float* orbit_out, bool orbit_only, const int32_t* __restrict__ g_orb,
            const float* __restrict__ norm_orb, uint32_t groups, uint32_t per_group) {
    // block b works on row block (b % groups) * per_group + b / groups; with
    // groups = the SM count, the blocks that start together on one SM take
    // neighbouring canonical rows, whose orbit rows overlap (L1 reuse);
    // groups = 1 is the plain order
    const uint32_t rb = (blockIdx.x % groups) * per_group + blockIdx.x / groups;
    const uint32_t row = rb * (blockDim.x >> 5) + (threadIdx.x >> 5);
    const uint32_t lane = threadIdx.x & 31u;
    if (row >= nrows) return;  // warp-uniform
    const uint32_t lb = lane & 3u, mg = lane & 1u, slot = lane >> 2;
    float acc[4] = {0.f, 0.f, 0.f, 0.f};
    const uint64_t* rp = rowptr4 + 4 * (uint64_t)row;
    const uint64_t r0 = rp[0], r1 = rp[1], r2 = rp[2], r3 = rp[3], r4 = rp[4];
    if (lane == 0 && r4 > r0) {
        // the row's keys and values into L2 ahead of the loads (16-byte
        // granules; the arrays are padded by 16 elements past their end)
        l2_prefetch_range(key + r0, (r4 - r0) * sizeof(uint32_t));
        l2_prefetch_range(val + r0, (r4 - r0) * sizeof(V));
    }
    orbit_segment<V, U, 0>(key, val, orb, r0, r1, slot, lb, mg, acc);
    orbit_segment<V, U, 1>(key, val, orb, r1, r2, slot, lb, mg, acc);
    orbit_segment<V, U, 2>(key, val, orb, r2, r3, slot, lb, mg, acc);
    orbit_segment<V, U, 3>(key, val, orb, r3, r4, slot, lb, mg, acc);
#pragma unroll
    for (int o = 4; o < 32; o <<= 1)
#pragma unroll
        for (int q = 0; q < 4; ++q) acc[q] += __shfl_xor_sync(0xffffffffu, acc[q], o);
    // lane s (< 16) takes the total of s = 4 (mg + 2 fg) + q from lane s >> 2
    const uint32_t sl = lane & 15u, src = sl >> 2, q = sl & 3u;
    const float b0 = __shfl_sync(0xffffffffu, acc[0], src), b1 = __shfl_sync(0xffffffffu, acc[1], src);
    const float b2 = __shfl_sync(0xffffffffu, acc[2], src), b3 = __shfl_sync(0xffffffffu, acc[3], src);
    const float mine = q == 0 ? b0 : (q == 1 ? b1 : (q == 2 ? b2 : b3));
    const uint64_t o16 = 16 * (uint64_t)row + lane;
    // lane s < 16: the first transformation with the same output row as s
    // (itself for the rows it writes); lanes 16-31 point at themselves
    const uint32_t leader = lane < 16 ? (uint32_t)(olead[row] >> (4 * lane)) & 15u : lane;
    if (orbit_only) {
        // MLEM loop of two compact projections: per-row operands and results
        // in orbit order (64 contiguous bytes per row), natural order only for
        // the optional forward projection
        const uint32_t r = (lane < 16 && fwproj) ? oimg[o16] : 0u;
        float res = mine;
        if (lane < 16) {
            if (EPI == (int)Epi::Correl) {
                res = (mine != 0.0f) ? __fdiv_rn((float)g_orb[o16], mine) : 0.0f;
            } else if (EPI == (int)Epi::Update) {
                const float tt = __fmul_rn(orbit_out[o16], mine);
                const float nn = norm_orb[o16];
                res = (nn == 0.0f) ? tt : __fdiv_rn(tt, nn);
            }
        }
        // duplicates take the value of the first s with the same output row
        const float v = __shfl_sync(0xffffffffu, res, leader);
        if (lane < 16) {
            orbit_out[o16] = v;
            if (EPI == (int)Epi::Correl && fwproj && leader == lane) fwproj[r] = mine;
        }
        return;
    }
    const uint32_t r = lane < 16 ? oimg[o16] : 0u;
    const bool writer = lane < 16 && leader == lane;
    float res = mine;
    if (writer) {
        if (EPI == (int)Epi::Correl) {
            res = (mine != 0.0f) ? __fdiv_rn((float)g[r], mine) : 0.0f;
            out[r] = res;
            if (fwproj) fwproj[r] = mine;
        } else if (EPI == (int)Epi::Update) {
            const float tt = __fmul_rn(f[r], mine);
            const float nn = norm[r];
            res = (nn == 0.0f) ? tt : __fdiv_rn(tt, nn);
            f[r] = res;
        } else {
            out[r] = res;
        }
    }
    if (orbit_out) {
        // every s gets the value written for its output row (by the first s
        // with that row), so the orbit array equals a gather of the output
        const float v = __shfl_sync(0xffffffffu, res, leader);
        if (lane < 16) orbit_out[o16] = v;
    }
}

// orb[i] = src[table[i]] for int32 (the sinogram in orbit order).
__global__ void k_orbit_gather_i32(int32_t* __restrict__ orb, const int32_t* __restrict__ src,
                                   const uint32_t* __restrict__ table, uint64_t n) {
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x)
        orb[i] = __ldg(src + __ldg(table + i));
}

// dst[table[i]] = orb[i] for every i that is its own leader (orbit order
// back to natural order; every natural element has exactly one leader).
__global__ void k_orbit_scatter(float* __restrict__ dst, const float* __restrict__ orb,
                                const uint32_t* __restrict__ table, const uint64_t* __restrict__ lead, uint64_t n) {
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
        const uint32_t sidx = (uint32_t)(i & 15u);
        if (((lead[i >> 4] >> (4 * sidx)) & 15u) == sidx) dst[table[i]] = orb[i];
    }
}

// orb[i] = src[table[i]]: the input vector in orbit order.
__global__ void k_orbit_gather(float* __restrict__ orb, const float* __restrict__ src,
                               const uint32_t* __restrict__ table, uint64_t n) {
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x)
        orb[i] = __ldg(src + __ldg(table + i));
}

// ---------------------------------------------------------------- build kernels
// Row lengths of A^ (natural LOR order): every row has its canonical row's length.
__global__ void k_sym_lens(const uint64_t* __restrict__ crp, const uint32_t* __restrict__ can_row, uint64_t nlor,
                           uint32_t* __restrict__ len) {
    for (uint64_t r = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; r < nlor; r += (uint64_t)gridDim.x * blockDim.x) {
        const uint32_t k = can_row[r];
        len[r] = (uint32_t)(crp[k + 1] - crp[k]);
    }
}

// Row r of A^ (unsorted) = canonical row can_row[r] with columns mapped by sym_of[r].
__global__ void k_sym_expand(const uint64_t* __restrict__ crp, const uint32_t* __restrict__ ccol,
                             const float* __restrict__ cval, const uint32_t* __restrict__ can_row,
                             const uint8_t* __restrict__ sym_of, uint64_t nlor, uint32_t n, uint32_t nz,
                             const uint64_t* __restrict__ orp, uint32_t* __restrict__ ocol, float* __restrict__ oval) {
    const uint32_t lane = threadIdx.x & 31;
    for (uint64_t r = (blockIdx.x * (uint64_t)blockDim.x + threadIdx.x) >> 5; r < nlor;
         r += ((uint64_t)gridDim.x * blockDim.x) >> 5) {
        const uint32_t k = can_row[r];
        const VoxMap m = vox_map(sym_of[r], (int32_t)n, (int32_t)nz);
        const uint64_t s = crp[k], len = crp[k + 1] - s, o = orp[r];
        for (uint64_t t = lane; t < len; t += 32) {
            const uint32_t c = ccol[s + t];
            const uint32_t xx = c % n, yy = (c / n) % n, zz = c / (n * n);
            ocol[o + t] = (uint32_t)(m.ax * (int32_t)xx + m.ay * (int32_t)yy + m.az * (int32_t)zz + m.c0);
            oval[o + t] = cval[s + t];
        }
    }
}

// Compact operands from CSR rows (row j of the output = input row rowsel[j],
// or j without a selection): an entry with column c becomes
// orb_of[c] << 4 | sym[c], and every output row is split into 4 segments by
// the rotation class sym[c] & 3 (stable inside a segment).  One warp per row.
__global__ void k_seg_counts(const uint64_t* __restrict__ rp, const uint32_t* __restrict__ idx,
                             const uint32_t* __restrict__ rowsel, uint32_t nrows, const uint8_t* __restrict__ sym,
                             uint32_t* __restrict__ counts) {
    const uint32_t lane = threadIdx.x & 31u;
    for (uint64_t j = (blockIdx.x * (uint64_t)blockDim.x + threadIdx.x) >> 5; j < nrows;
         j += ((uint64_t)gridDim.x * blockDim.x) >> 5) {
        const uint32_t r = rowsel ? rowsel[j] : (uint32_t)j;
        uint32_t c[4] = {0, 0, 0, 0};
        for (uint64_t e = rp[r] + lane; e < rp[r + 1]; e += 32) {
            const uint32_t q = sym[idx[e]] & 3u;
            c[0] += q == 0;
            c[1] += q == 1;
            c[2] += q == 2;
            c[3] += q == 3;
        }
#pragma unroll
        for (int q = 0; q < 4; ++q)
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) c[q] += __shfl_xor_sync(0xffffffffu, c[q], o);
        if (lane < 4) counts[4 * j + lane] = c[0] * (lane == 0) + c[1] * (lane == 1) + c[2] * (lane == 2) + c[3] * (lane == 3);
    }
}

__global__ void k_seg_fill(const uint64_t* __restrict__ rp, const uint32_t* __restrict__ idx,
                           const float* __restrict__ val, const uint32_t* __restrict__ rowsel, uint32_t nrows,
                           const uint32_t* __restrict__ orb_of, const uint8_t* __restrict__ sym,
                           const uint64_t* __restrict__ orp, uint32_t* __restrict__ okey, float* __restrict__ oval) {
    const uint32_t lane = threadIdx.x & 31u;
    for (uint64_t j = (blockIdx.x * (uint64_t)blockDim.x + threadIdx.x) >> 5; j < nrows;
         j += ((uint64_t)gridDim.x * blockDim.x) >> 5) {
        const uint32_t r = rowsel ? rowsel[j] : (uint32_t)j;
        const uint64_t s0 = rp[r], s1 = rp[r + 1];
        for (uint32_t q = 0; q < 4; ++q) {
            uint64_t o = orp[4 * j + q];
            for (uint64_t base = s0; base < s1; base += 32) {
                const uint64_t e = base + lane;
                uint32_t c = 0, t = 0;
                bool take = false;
                if (e < s1) {
                    c = idx[e];
                    t = sym[c];
                    take = (t & 3u) == q;
                }
                const uint32_t b = __ballot_sync(0xffffffffu, take);
                if (take) {
                    const uint64_t pos = o + __popc(b & ((1u << lane) - 1u));
                    okey[pos] = (orb_of[c] << 4) | t;
                    oval[pos] = val[e];
                }
                o += __popc(b);
            }
        }
    }
}

// Each segment sorted by key (orbit row, then transformation), so the entries
// one load instruction covers tend to share 128-byte orbit lines.  One warp
// per segment, bitonic in shared memory; segments longer than kSortCap stay
// in column order (the order does not change the sums beyond rounding).
constexpr uint32_t kSortCap = 2048;

__global__ void k_seg_sort(const uint64_t* __restrict__ orp, uint64_t nseg, uint32_t* __restrict__ key,
                           float* __restrict__ val) {
    extern __shared__ __align__(16) unsigned char sm[];
    const uint32_t lane = threadIdx.x & 31u, w = threadIdx.x >> 5;
    uint32_t* sk = reinterpret_cast<uint32_t*>(sm) + (size_t)w * kSortCap * 2;
    float* sv = reinterpret_cast<float*>(sk + kSortCap);
    for (uint64_t g = (blockIdx.x * (uint64_t)blockDim.x + threadIdx.x) >> 5; g < nseg;
         g += ((uint64_t)gridDim.x * blockDim.x) >> 5) {
        const uint64_t s0 = orp[g], n = orp[g + 1] - s0;
        if (n < 2 || n > kSortCap) continue;  // warp-uniform
        uint32_t m = 32;
        while (m < n) m <<= 1;
        for (uint32_t i = lane; i < m; i += 32) {
            sk[i] = i < n ? key[s0 + i] : 0xffffffffu;
            sv[i] = i < n ? val[s0 + i] : 0.f;
        }
        __syncwarp();
        for (uint32_t k = 2; k <= m; k <<= 1)
            for (uint32_t j = k >> 1; j > 0; j >>= 1) {
                for (uint32_t i = lane; i < m; i += 32) {
                    const uint32_t p = i ^ j;
                    if (p > i) {
                        const bool up = (i & k) == 0;
                        if ((sk[i] > sk[p]) == up) {
                            const uint32_t tk = sk[i];
                            sk[i] = sk[p];
                            sk[p] = tk;
                            const float tv = sv[i];
                            sv[i] = sv[p];
                            sv[p] = tv;
                        }
                    }
                }
                __syncwarp();
            }
        for (uint32_t i = lane; i < n; i += 32) {
            key[s0 + i] = sk[i];
            val[s0 + i] = sv[i];
        }
        __syncwarp();
    }
}

// Builds one compact operand (segmented row pointers [4 nrows + 1], keys, FP32 values).
void build_segmented(const uint64_t* rp, const uint32_t* idx, const float* val, const uint32_t* rowsel, uint32_t nrows,
                     const uint32_t* orb_of, const uint8_t* sym, uint64_t*& orp, uint32_t*& okey, void*& oval,
                     uint64_t& onnz, cudaStream_t s);

unsigned grid_of(uint64_t n) { return std::max(1u, std::min<unsigned>(ceil_div_u(n, 256), 152u * 32u)); }

template <typename T>
T* upload(const std::vector<T>& h, size_t min_elems = 1) {
    T* d = nullptr;
    MLEM_CUDA(cudaMalloc(&d, sizeof(T) * std::max(h.size(), min_elems)));
    if (!h.empty()) MLEM_CUDA(cudaMemcpy(d, h.data(), sizeof(T) * h.size(), cudaMemcpyHostToDevice));
    return d;
}

void build_segmented(const uint64_t* rp, const uint32_t* idx, const float* val, const uint32_t* rowsel, uint32_t nrows,
                     const uint32_t* orb_of, const uint8_t* sym, uint64_t*& orp, uint32_t*& okey, void*& oval,
                     uint64_t& onnz, cudaStream_t s) {
    const uint64_t nseg = 4ull * nrows;
    uint32_t* counts = nullptr;
    MLEM_CUDA(cudaMalloc(&counts, sizeof(uint32_t) * std::max<uint64_t>(nseg, 1)));
    try {
        MLEM_CUDA(cudaMalloc(&orp, sizeof(uint64_t) * (nseg + 1)));
        k_seg_counts<<<grid_of((uint64_t)nrows * 32), 256, 0, s>>>(rp, idx, rowsel, nrows, sym, counts);
        MLEM_LAUNCHED();
        scan_counts_u64(counts, orp, nseg, s);
        MLEM_CUDA(cudaMemcpyAsync(&onnz, orp + nseg, sizeof(uint64_t), cudaMemcpyDeviceToHost, s));
        MLEM_CUDA(cudaStreamSynchronize(s));
        // 16 elements of padding: the kernels prefetch whole 16-byte granules
        MLEM_CUDA(cudaMalloc(&okey, sizeof(uint32_t) * (onnz + 16)));
        MLEM_CUDA(cudaMalloc(&oval, sizeof(float) * (onnz + 16)));
        k_seg_fill<<<grid_of((uint64_t)nrows * 32), 256, 0, s>>>(rp, idx, val, rowsel, nrows, orb_of, sym, orp, okey,
                                                                   static_cast<float*>(oval));
        MLEM_LAUNCHED();
        constexpr int kSortWarps = 4;
        const size_t smem = (size_t)kSortWarps * kSortCap * 8;
        MLEM_CUDA(cudaFuncSetAttribute(k_seg_sort, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        k_seg_sort<<<grid_of(nseg * 32 / 2), kSortWarps * 32, smem, s>>>(orp, nseg, okey, static_cast<float*>(oval));
        MLEM_LAUNCHED();
        MLEM_CUDA(cudaStreamSynchronize(s));
    } catch (...) {
        cudaFree(counts);
        throw;
    }
    cudaFree(counts);
}

template <typename V, int EPI, int U>
void orbit_launch(const SymOps& y, bool transposed, const float* x, const EpiArgs& e, bool grouped, L2Window win,
                  cudaStream_t s) {
    const uint32_t rows = transposed ? y.J : y.K;
    float* orb = transposed ? y.orb_r : y.orb_x;
    const uint32_t* table = transposed ? y.img : y.vimg;  // input orbits: LORs for BP, voxels for FP
    const uint64_t n_orb = 16ull * (transposed ? y.K : y.J);
    if (!e.orbit_ready) {
        k_orbit_gather<<<grid_of(n_orb), 256, 0, s>>>(orb, x, table, n_orb);
        MLEM_LAUNCHED();
    }
    // the kernel gathers from the orbit array, not from x: an L2 window, if
    // asked for, covers that
    if (win.ptr) win = {orb, sizeof(float) * n_orb};
    const uint32_t row_blocks = (uint32_t)ceil_div_u((uint64_t)rows * 32, kOrbitBlock);
    const uint32_t groups = grouped ? 152u : 1u, per_group = (uint32_t)ceil_div_u(row_blocks, groups);
    launch_ex(k_sym_orbit<V, EPI, U>, dim3(groups * per_group), dim3(kOrbitBlock), 0, s, win,
              transposed ? y.bp_rowptr : y.fp_rowptr, transposed ? y.bp_key : y.fp_key,
              static_cast<const V*>(transposed ? y.bp_val : y.fp_val), rows, reinterpret_cast<const float4*>(orb),
              transposed ? y.vimg : y.img, transposed ? y.vlead : y.lead, e.g, e.out, e.fwproj, e.f, e.norm,
              e.orbit_out, e.orbit_only, y.g_orb, y.norm_orb, groups, per_group);
}

template <typename V, int EPI>
void orbit_variant(const SymOps& y, bool transposed, const float* x, const EpiArgs& e, int unroll, bool grouped,
                   L2Window win, cudaStream_t s) {
    if (unroll >= 8) orbit_launch<V, EPI, 8>(y, transposed, x, e, grouped, win, s);
    else if (unroll >= 4) orbit_launch<V, EPI, 4>(y, transposed, x, e, grouped, win, s);
    else orbit_launch<V, EPI, 2>(y, transposed, x, e, grouped, win, s);
}

template <typename V>
void sym_dispatch(const SymOps& y, bool transposed, const float* x, const EpiArgs& e, int unroll, bool grouped,
                  L2Window win, cudaStream_t s) {
    if (!transposed) {
        if (e.kind == Epi::Correl) orbit_variant<V, (int)Epi::Correl>(y, false, x, e, unroll, grouped, win, s);
        else orbit_variant<V, (int)Epi::Raw>(y, false, x, e, unroll, grouped, win, s);
    } else {
        if (e.kind == Epi::Update) orbit_variant<V, (int)Epi::Update>(y, true, x, e, unroll, grouped, win, s);
        else orbit_variant<V, (int)Epi::Raw>(y, true, x, e, unroll, grouped, win, s);
    }
}

}  // namespace

void SymOps::release() {
    cudaFree(fp_rowptr);
    cudaFree(fp_key);
    cudaFree(fp_val);
    cudaFree(img);
    cudaFree(lead);
    cudaFree(bp_rowptr);
    cudaFree(bp_key);
    cudaFree(bp_val);
    cudaFree(vimg);
    cudaFree(vlead);
    cudaFree(norm_orb);
    cudaFree(g_orb);
    cudaFree(orb_x);
    cudaFree(orb_r);
    *this = SymOps();
}

uint64_t SymOps::bytes() const {
    if (!fp_rowptr) return 0;
    const size_t vb = val_bytes(vt);
    // row pointers, entries, and per canonical row / voxel: 16 images, a
    // leader word, 2 orbit arrays (image or ratio, plus sinogram or sensitivity)
    return sizeof(uint64_t) * (4 * ((uint64_t)K + J) + 2) + (4 + vb) * (fp_nnz + bp_nnz) +
           (16 * 4 + 8 + 2 * 16 * 4) * ((uint64_t)K + J);
}

void check_symmetric_geometry(const mlem_geometry& g) {
    MLEM_REQUIRE(g.nx == g.ny, MLEM_EUNSUPPORTED, "symmetry needs a square voxel grid (nx == ny)");
    MLEM_REQUIRE(g.det_per_ring % 4 == 0, MLEM_EUNSUPPORTED, "symmetry needs a multiple of 4 detectors per ring");
    MLEM_REQUIRE(g.row_stride <= 1, MLEM_EUNSUPPORTED, "symmetry needs every LOR (row_stride 1)");
    MLEM_REQUIRE(g.vx == g.vy, MLEM_EUNSUPPORTED, "symmetry needs square voxels in the transaxial plane");
}

namespace {

// The rows of the given canonical LORs (host CSR over the full column range).
using CanonicalRows = std::function<void(const std::vector<uint64_t>& lors, std::vector<uint64_t>& rowptr,
                                         std::vector<uint32_t>& col, std::vector<float>& val)>;

// A^ from the canonical rows that rows_of supplies (averaged over the
// transformations that fix their LOR), its transpose and the compact operands.
void build_symmetric_impl(const SymMaps& M, const CanonicalRows& rows_of, DevCsr& A, DevCsr& AT, SymOps& y,
                          cudaStream_t s) {
    const uint64_t D = M.D, nlor = D * (D - 1) / 2, cols = (uint64_t)M.n * M.n * M.nz;
    MLEM_REQUIRE(nlor < (1ull << 32), MLEM_EUNSUPPORTED, "symmetry: too many LORs");
    uint8_t comp[16][16], inv[16];
    composition(M, comp, inv);

    // LOR orbits: canonical rows (smallest index of each orbit) and, for every
    // LOR, its canonical row and the first transformation that produces it
    std::vector<uint8_t> canon_flag(nlor, 0);
#pragma omp parallel for schedule(dynamic, 16)
    for (int64_t a = 0; a < (int64_t)D - 1; ++a) {
        for (uint64_t b = (uint64_t)a + 1; b < D; ++b) {
            const uint64_t r = M.lor((uint64_t)a, b);
            uint64_t mn = r;
            for (int t = 1; t < 16; ++t) mn = std::min<uint64_t>(mn, M.lor(M.det(t, (uint32_t)a), M.det(t, (uint32_t)b)));
            canon_flag[r] = mn == r;
        }
    }
    std::vector<uint64_t> canon;
    std::vector<uint32_t> pair_a;
    for (uint64_t a = 0; a + 1 < D; ++a)
        for (uint64_t b = a + 1; b < D; ++b)
            if (canon_flag[M.lor(a, b)]) {
                canon.push_back(M.lor(a, b));
                pair_a.push_back((uint32_t)a);
            }
    std::vector<uint8_t>().swap(canon_flag);
    const uint64_t K = canon.size();
    MLEM_REQUIRE(K < (1ull << 28), MLEM_EUNSUPPORTED, "symmetry: too many canonical rows");
    std::vector<uint32_t> img(16 * K), can_row(nlor);
    std::vector<uint64_t> lead(K, 0);
    std::vector<uint8_t> sym_of(nlor);
#pragma omp parallel for schedule(static)
    for (int64_t k = 0; k < (int64_t)K; ++k) {
        const uint64_t r = canon[k];
        const uint32_t a = pair_a[k], b = (uint32_t)(r - M.lor(a, a + 1) + a + 1);
        for (int t = 0; t < 16; ++t) {
            const uint64_t im = M.lor(M.det(t, a), M.det(t, b));
            img[16 * k + t] = (uint32_t)im;
            int first = 0;
            while (img[16 * k + first] != im) ++first;
            lead[k] |= (uint64_t)first << (4 * t);
            if (first == t) {
                can_row[im] = (uint32_t)k;
                sym_of[im] = (uint8_t)t;
            }
        }
    }
    // voxel orbits: canonical voxels (smallest index of each orbit), their 16
    // images, and for every voxel its canonical voxel and the first
    // transformation that produces it
    std::vector<uint32_t> vrow, vimg, vorb(cols);
    std::vector<uint64_t> vlead;
    std::vector<uint8_t> vsym(cols);
    for (uint32_t c = 0; c < cols; ++c) {
        uint32_t seen[16];
        uint32_t mn = c;
        for (int t = 0; t < 16; ++t) mn = std::min(mn, seen[t] = M.vox_index(t, c));
        if (mn != c) continue;
        const uint32_t j = (uint32_t)vrow.size();
        uint64_t ld = 0;
        for (int t = 0; t < 16; ++t) {
            int first = 0;
            while (seen[first] != seen[t]) ++first;
            ld |= (uint64_t)first << (4 * t);
            if (first == t) {
                vorb[seen[t]] = j;
                vsym[seen[t]] = (uint8_t)t;
            }
            vimg.push_back(seen[t]);
        }
        vrow.push_back(c);
        vlead.push_back(ld);
    }
    MLEM_REQUIRE(vrow.size() < (1ull << 28), MLEM_EUNSUPPORTED, "symmetry: too many canonical voxels");

    // canonical rows, averaged over the transformations that fix their LOR
    std::vector<uint64_t> crp;
    std::vector<uint32_t> ccol;
    std::vector<float> cval;
    rows_of(canon, crp, ccol, cval);
    {
        std::vector<uint64_t> nrp(K + 1, 0);
        std::vector<uint32_t> ncol;
        std::vector<float> nval;
        ncol.reserve(ccol.size());
        nval.reserve(cval.size());
        for (uint64_t k = 0; k < K; ++k) {
            const uint64_t r = canon[k];
            int H[16], nh = 0;
            for (int t = 0; t < 16; ++t)
                if (img[16 * k + t] == r) H[nh++] = t;
            if (nh == 1) {
                for (uint64_t e = crp[k]; e < crp[k + 1]; ++e) {
                    ncol.push_back(ccol[e]);
                    nval.push_back(cval[e]);
                }
            } else {
                std::map<uint32_t, float> orig;
                for (uint64_t e = crp[k]; e < crp[k + 1]; ++e) orig[ccol[e]] = cval[e];
                std::map<uint32_t, double> sym;
                for (const auto& kv : orig)
                    for (int h = 0; h < nh; ++h) sym[M.vox_index(H[h], kv.first)] = 0.0;
                for (auto& kv : sym) {
                    double acc = 0.0;
                    for (int h = 0; h < nh; ++h) {
                        auto it = orig.find(M.vox_index(inv[H[h]], kv.first));
                        if (it != orig.end()) acc += it->second;
                    }
                    kv.second = acc / nh;
                }
                for (const auto& kv : sym) {
                    ncol.push_back(kv.first);
                    nval.push_back((float)kv.second);
                }
            }
            nrp[k + 1] = ncol.size();
        }
        crp.swap(nrp);
        ccol.swap(ncol);
        cval.swap(nval);
    }
    const uint64_t cnnz = crp[K];

    // device: canonical rows, then A^ (every LOR) by expansion and two stable transposes
    uint64_t* d_crp = nullptr;
    uint32_t *d_ccol = nullptr, *d_can = nullptr, *len = nullptr;
    float* d_cval = nullptr;
    uint8_t* d_sym = nullptr;
    DevCsr R;
    try {
        d_crp = upload(crp);
        d_ccol = upload(ccol);
        d_cval = upload(cval);
        d_can = upload(can_row);
        d_sym = upload(sym_of);
        R.nrows = (uint32_t)nlor;
        R.ncols = (uint32_t)cols;
        R.vt = MLEM_VAL_F32;
        MLEM_CUDA(cudaMalloc(&len, sizeof(uint32_t) * std::max<uint64_t>(nlor, 1)));
        k_sym_lens<<<grid_of(nlor), 256, 0, s>>>(d_crp, d_can, nlor, len);
        MLEM_LAUNCHED();
        MLEM_CUDA(cudaMalloc(&R.rowptr, sizeof(uint64_t) * (nlor + 1)));
        scan_counts_u64(len, R.rowptr, nlor, s);
        MLEM_CUDA(cudaMemcpyAsync(&R.nnz, R.rowptr + nlor, sizeof(uint64_t), cudaMemcpyDeviceToHost, s));
        MLEM_CUDA(cudaStreamSynchronize(s));
        MLEM_CUDA(cudaMalloc(&R.idx, sizeof(uint32_t) * padded(R.nnz)));
        MLEM_CUDA(cudaMalloc(&R.val, sizeof(float) * padded(R.nnz)));
        MLEM_CUDA(cudaMemsetAsync(R.idx, 0, sizeof(uint32_t) * padded(R.nnz), s));
        MLEM_CUDA(cudaMemsetAsync(R.val, 0, sizeof(float) * padded(R.nnz), s));
        k_sym_expand<<<grid_of(nlor * 32), 256, 0, s>>>(d_crp, d_ccol, d_cval, d_can, d_sym, nlor, M.n, M.nz,
                                                         R.rowptr, R.idx, static_cast<float*>(R.val));
        MLEM_LAUNCHED();
        transpose_device(R, AT, s);  // voxel rows, LORs ascending: the transpose of A^
        MLEM_CUDA(cudaStreamSynchronize(s));
        cudaFree(R.rowptr);
        cudaFree(R.idx);
        cudaFree(R.val);
        R = DevCsr();
        transpose_device(AT, A, s);  // A^, columns ascending in every row
        A.max_row = max_row_length(A.rowptr, A.nrows, s);

        // forward-projection operand: the canonical rows, columns as canonical voxel << 4 | t
        y.K = (uint32_t)K;
        y.J = (uint32_t)vrow.size();
        {
            uint32_t* d_vorb = upload(vorb);
            uint8_t* d_vsym = upload(vsym);
            try {
                build_segmented(d_crp, d_ccol, d_cval, nullptr, y.K, d_vorb, d_vsym, y.fp_rowptr, y.fp_key, y.fp_val,
                                y.fp_nnz, s);
            } catch (...) {
                cudaFree(d_vorb);
                cudaFree(d_vsym);
                throw;
            }
            cudaFree(d_vorb);
            cudaFree(d_vsym);
        }
        y.img = upload(img);
        y.lead = upload(lead);
        // back-projection operand: rows of A^T for the canonical voxels, LORs as canonical row << 4 | t
        {
            uint32_t* d_vrow = upload(vrow);
            try {
                build_segmented(AT.rowptr, AT.idx, static_cast<const float*>(AT.val), d_vrow, y.J, d_can, d_sym,
                                y.bp_rowptr, y.bp_key, y.bp_val, y.bp_nnz, s);
            } catch (...) {
                cudaFree(d_vrow);
                throw;
            }
            cudaFree(d_vrow);
        }
        y.vimg = upload(vimg);
        y.vlead = upload(vlead);
        MLEM_CUDA(cudaMalloc(&y.norm_orb, sizeof(float) * 16 * std::max<uint64_t>(y.J, 1)));
        MLEM_CUDA(cudaMalloc(&y.g_orb, sizeof(int32_t) * 16 * std::max<uint64_t>(y.K, 1)));
        MLEM_CUDA(cudaMalloc(&y.orb_x, sizeof(float) * 16 * std::max<uint64_t>(y.J, 1)));
        MLEM_CUDA(cudaMalloc(&y.orb_r, sizeof(float) * 16 * std::max<uint64_t>(y.K, 1)));
        y.vt = MLEM_VAL_F32;
    } catch (...) {
        cudaStreamSynchronize(s);
        cudaFree(d_crp);
        cudaFree(d_ccol);
        cudaFree(d_cval);
        cudaFree(d_can);
        cudaFree(d_sym);
        cudaFree(len);
        cudaFree(R.rowptr);
        cudaFree(R.idx);
        cudaFree(R.val);
        throw;
    }
    cudaFree(d_crp);
    cudaFree(d_ccol);
    cudaFree(d_cval);
    cudaFree(d_can);
    cudaFree(d_sym);
    cudaFree(len);
}

__global__ void k_count_diff(const uint32_t* __restrict__ a, const uint32_t* __restrict__ b, uint64_t n,
                             unsigned long long* __restrict__ count) {
    unsigned long long local = 0;
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x)
        local += a[i] != b[i];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) local += __shfl_xor_sync(0xffffffffu, local, o);
    if ((threadIdx.x & 31) == 0 && local) atomicAdd(count, local);
}

// Words that differ between two device arrays of n 32-bit words.
uint64_t count_diff(const void* a, const void* b, uint64_t n, cudaStream_t s) {
    if (n == 0) return 0;
    unsigned long long* d = nullptr;
    MLEM_CUDA(cudaMalloc(&d, sizeof(unsigned long long)));
    unsigned long long h = 0;
    cudaError_t e = cudaMemsetAsync(d, 0, sizeof(unsigned long long), s);
    if (e == cudaSuccess) {
        k_count_diff<<<grid_of(n), 256, 0, s>>>(static_cast<const uint32_t*>(a), static_cast<const uint32_t*>(b), n, d);
        count_launch();
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaMemcpyAsync(&h, d, sizeof(h), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    cudaFree(d);
    MLEM_CUDA(e);
    return h;
}

SymMaps maps_of(uint32_t n, uint32_t nz, uint32_t dpr, uint32_t rings) {
    SymMaps M;
    M.n = n;
    M.nz = nz;
    M.dpr = dpr;
    M.rings = rings;
    M.D = dpr * rings;
    return M;
}

}  // namespace

void build_symmetric(const mlem_geometry& geo, DevCsr& A, DevCsr& AT, SymOps& y, cudaStream_t s) {
    check_symmetric_geometry(geo);
    build_symmetric_impl(
        maps_of(geo.nx, geo.nz, geo.det_per_ring, geo.n_rings),
        [&](const std::vector<uint64_t>& lors, std::vector<uint64_t>& rp, std::vector<uint32_t>& col,
            std::vector<float>& val) { siddon_rows_of_lors(geo, lors, rp, col, val); },
        A, AT, y, s);
}

void build_symmetric_checked(const mlem_csr_host& c, const DevCsr& user, uint32_t n, uint32_t nz, uint32_t dpr,
                             uint32_t rings, DevCsr& A, DevCsr& AT, SymOps& y, cudaStream_t s) {
    MLEM_REQUIRE(n >= 1 && nz >= 1, MLEM_EINVAL, "symmetry: grid_nx and grid_nz must be given");
    MLEM_REQUIRE(dpr >= 4 && dpr % 4 == 0 && rings >= 1, MLEM_EUNSUPPORTED,
                 "symmetry: needs a ring scanner with a multiple of 4 detectors per ring (sym_det_per_ring)");
    const uint64_t D = (uint64_t)dpr * rings;
    MLEM_REQUIRE(D <= 16384, MLEM_EUNSUPPORTED, "symmetry: too many detectors");
    MLEM_REQUIRE((uint64_t)c.rows == D * (D - 1) / 2, MLEM_EINVAL,
                 "symmetry: the rows must be the " + std::to_string(D * (D - 1) / 2) +
                     " detector pairs (a < b, lexicographic) of the scanner");
    MLEM_REQUIRE((uint64_t)c.cols == (uint64_t)n * n * nz, MLEM_EINVAL,
                 "symmetry: the columns must be the grid_nx x grid_nx x grid_nz voxels");
    build_symmetric_impl(
        maps_of(n, nz, dpr, rings),
        [&](const std::vector<uint64_t>& lors, std::vector<uint64_t>& rp, std::vector<uint32_t>& col,
            std::vector<float>& val) {
            rp.assign(lors.size() + 1, 0);
            for (size_t k = 0; k < lors.size(); ++k) rp[k + 1] = rp[k] + (c.rowptr[lors[k] + 1] - c.rowptr[lors[k]]);
            col.resize(rp.back());
            val.resize(rp.back());
            for (size_t k = 0; k < lors.size(); ++k) {
                const uint64_t b = c.rowptr[lors[k]], e = c.rowptr[lors[k] + 1];
                std::memcpy(col.data() + rp[k], c.col + b, sizeof(uint32_t) * (e - b));
                std::memcpy(val.data() + rp[k], c.val + b, sizeof(float) * (e - b));
            }
        },
        A, AT, y, s);
    // A^ was built from the canonical rows alone; it equals the caller's
    // matrix bit for bit exactly when that matrix is invariant under the 16
    // transformations (with every row's columns ascending).
    uint64_t diff = A.nnz == user.nnz ? 0 : ~0ull;
    if (diff == 0) diff = count_diff(A.rowptr, user.rowptr, 2 * ((uint64_t)A.nrows + 1), s);
    if (diff == 0) diff = count_diff(A.idx, user.idx, A.nnz, s) + count_diff(A.val, user.val, A.nnz, s);
    if (diff != 0) {
        fail(MLEM_EINVAL,
             "symmetry: the matrix is not invariant under the 16 symmetries of the scanner (" +
                 (A.nnz == user.nnz ? std::to_string(diff) + " words differ from"
                                    : std::string("its nonzero count differs from")) +
                 " the symmetric matrix built from its canonical rows; every row must list its columns in ascending "
                 "order)");
    }
}

void lower_symmetric_values(SymOps& y, mlem_value_type vt, cudaStream_t s) {
    if (vt == MLEM_VAL_F32 || !y.fp_rowptr) return;
    auto lower = [&](void*& v, uint64_t n) {
        void* nv = nullptr;
        MLEM_CUDA(cudaMalloc(&nv, 2 * (n + 16)));
        convert_values(static_cast<const float*>(v), nv, vt, n, s);
        MLEM_CUDA(cudaStreamSynchronize(s));
        cudaFree(v);
        v = nv;
    };
    lower(y.fp_val, y.fp_nnz);
    lower(y.bp_val, y.bp_nnz);
    y.vt = vt;
}

void sym_set_norm(SymOps& y, const float* norm, cudaStream_t s) {
    if (!y.fp_rowptr) return;
    const uint64_t n = 16ull * y.J;
    k_orbit_gather<<<grid_of(n), 256, 0, s>>>(y.norm_orb, norm, y.vimg, n);
    MLEM_LAUNCHED();
}

void sym_gather_sinogram(const SymOps& y, const int32_t* g, cudaStream_t s) {
    MLEM_REQUIRE(y.fp_rowptr != nullptr, MLEM_EINVAL, "matrix has no symmetry operands");
    const uint64_t n = 16ull * y.K;
    k_orbit_gather_i32<<<grid_of(n), 256, 0, s>>>(y.g_orb, g, y.img, n);
    MLEM_LAUNCHED();
}

void sym_scatter_image(const SymOps& y, float* f, cudaStream_t s) {
    MLEM_REQUIRE(y.fp_rowptr != nullptr, MLEM_EINVAL, "matrix has no symmetry operands");
    const uint64_t n = 16ull * y.J;
    k_orbit_scatter<<<grid_of(n), 256, 0, s>>>(f, y.orb_x, y.vimg, y.vlead, n);
    MLEM_LAUNCHED();
}

void sym_gather_image(const SymOps& y, const float* f, cudaStream_t s) {
    MLEM_REQUIRE(y.fp_rowptr != nullptr, MLEM_EINVAL, "matrix has no symmetry operands");
    const uint64_t n = 16ull * y.J;
    k_orbit_gather<<<grid_of(n), 256, 0, s>>>(y.orb_x, f, y.vimg, n);
    MLEM_LAUNCHED();
}

void launch_sym(const SymOps& y, bool transposed, const float* x, const EpiArgs& e, int unroll, bool grouped,
                L2Window win, cudaStream_t s) {
    MLEM_REQUIRE(y.fp_rowptr != nullptr, MLEM_EINVAL, "matrix has no symmetry operands");
    switch (y.vt) {
        case MLEM_VAL_F32: sym_dispatch<float>(y, transposed, x, e, unroll, grouped, win, s); break;
        case MLEM_VAL_F16: sym_dispatch<__half>(y, transposed, x, e, unroll, grouped, win, s); break;
        default: sym_dispatch<__nv_bfloat16>(y, transposed, x, e, unroll, grouped, win, s);
    }
}

}  // namespace mlem
