/*
 * siddon_oracle.c — CPU generator of the synthetic system matrices.
 *
 * TEST AND BENCHMARK INFRASTRUCTURE ONLY.  The product library has its own
 * generator (a __host__ __device__ routine run on the GPU or with OpenMP on
 * the host).  This file restates that generator in plain C so that the CPU
 * baseline of the benchmark (the reference arm) can build its inputs without
 * loading the product library; a CPU test checks that both produce the same
 * matrix bit for bit.
 *
 * The matrix: rows are the unordered detector pairs (a < b) of a cylindrical
 * ring scanner in lexicographic order (optionally every row_stride-th from
 * row_phase), columns are voxels x + nx*(y + ny*z) (the reference's numbering,
 * scannerconfig.cpp:30-35), values are the mean over sub_t x sub_z parallel
 * sub-rays across the crystal faces of the exact ray/voxel intersection
 * length (Siddon 1985: incremental traversal of the x/y/z plane crossings,
 * the voxel of each segment taken at its midpoint; consecutive segments in
 * one voxel merged; pieces of 1e-6 mm or shorter dropped).  Columns ascend
 * within a row.
 *
 * Floating point: double precision throughout, IEEE +,-,*,/, sqrt, floor,
 * ceil, fmin, fmax only; compiled with -ffp-contract=off.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

/* Same field layout as the library's mlem_geometry. */
typedef struct {
    uint32_t det_per_ring, n_rings;
    float radius, ring_pitch;
    uint32_t nx, ny, nz;
    float vx, vy, vz;
    uint32_t row_stride, row_phase;
    uint32_t sub_t, sub_z;
    float width_t, width_z;
} oracle_geometry;

typedef struct {
    uint32_t dpr, rings, D;
    double radius, pitch;
    uint32_t nx, ny, nz;
    double vx, vy, vz, x0, y0, z0;
    uint64_t nlor, stride, phase, nrows;
    uint32_t sub_t, sub_z, S;
    double width_t, width_z;
    uint32_t cap_ray;
    const double* ct;
    const double* st;
} Scan;

static const double kMinLen = 1e-6;

static int make_scan(const oracle_geometry* g, Scan* G) {
    if (g->det_per_ring < 1 || g->n_rings < 1) return -1;
    if ((uint64_t)g->det_per_ring * g->n_rings < 2 || (uint64_t)g->det_per_ring * g->n_rings > 16384) return -1;
    if (g->nx < 1 || g->ny < 1 || g->nz < 1) return -1;
    if ((uint64_t)g->nx * g->ny * g->nz >= (1ull << 32)) return -1;
    if (!(g->vx > 0 && g->vy > 0 && g->vz > 0 && g->radius > 0)) return -1;
    if (g->row_stride > 1 && g->row_phase >= g->row_stride) return -1;
    G->dpr = g->det_per_ring;
    G->rings = g->n_rings;
    G->D = g->det_per_ring * g->n_rings;
    G->radius = g->radius;
    G->pitch = g->ring_pitch;
    G->nx = g->nx;
    G->ny = g->ny;
    G->nz = g->nz;
    G->vx = g->vx;
    G->vy = g->vy;
    G->vz = g->vz;
    G->x0 = -0.5 * G->nx * G->vx;
    G->y0 = -0.5 * G->ny * G->vy;
    G->z0 = -0.5 * G->nz * G->vz;
    G->nlor = (uint64_t)G->D * (G->D - 1) / 2;
    G->stride = g->row_stride > 1 ? g->row_stride : 1;
    G->phase = g->row_stride > 1 ? g->row_phase : 0;
    G->nrows = G->nlor > G->phase ? (G->nlor - G->phase + G->stride - 1) / G->stride : 0;
    G->sub_t = g->sub_t > 1 ? g->sub_t : 1;
    G->sub_z = g->sub_z > 1 ? g->sub_z : 1;
    G->S = G->sub_t * G->sub_z;
    if (G->S > 32) return -1;
    G->width_t = g->width_t;
    G->width_z = g->width_z;
    G->cap_ray = g->nx + g->ny + g->nz + 8;
    return 0;
}

/* cos/sin of the detector angles 2*pi*k/dpr, exact zeros on the axes. */
static void angles(const Scan* G, double* ct, double* st) {
    const double two_pi = 6.283185307179586476925286766559;
    for (uint32_t k = 0; k < G->dpr; ++k) {
        const double th = two_pi * (double)k / (double)G->dpr;
        ct[k] = cos(th);
        st[k] = sin(th);
        if (fabs(ct[k]) < 1e-12) ct[k] = 0.0;
        if (fabs(st[k]) < 1e-12) st[k] = 0.0;
    }
}

/* first LOR index of detector a's pairs (a, b > a) */
static inline uint64_t first_lor(uint64_t a, uint64_t D) { return a * D - a * (a + 1) / 2; }

static void pair_of(uint64_t r, uint64_t D, uint32_t* a, uint32_t* b) {
    uint64_t lo = 0, hi = D - 2;
    while (lo < hi) {
        const uint64_t mid = (lo + hi + 1) >> 1;
        if (first_lor(mid, D) <= r) lo = mid;
        else hi = mid - 1;
    }
    *a = (uint32_t)lo;
    *b = (uint32_t)(r - first_lor(lo, D) + lo + 1);
}

static void detector(const Scan* G, uint32_t d, double* x, double* y, double* z) {
    const uint32_t ring = d / G->dpr, k = d % G->dpr;
    *x = G->radius * G->ct[k];
    *y = G->radius * G->st[k];
    *z = ((double)ring - 0.5 * (double)(G->rings - 1)) * G->pitch;
}

/* sub-ray k of LOR (a, b): tangential offset u and axial offset v across the
 * crystal faces, mirrored at b so facing sub-rays are parallel */
static void subray(const Scan* G, uint32_t a, uint32_t b, uint32_t k, double p[6]) {
    const uint32_t i = k % G->sub_t, j = k / G->sub_t;
    const double u = ((double)i + 0.5) / (double)G->sub_t - 0.5;
    const double v = (((double)j + 0.5) / (double)G->sub_z - 0.5) * G->width_z;
    const double ut = u * G->width_t;
    const uint32_t ka = a % G->dpr, kb = b % G->dpr;
    detector(G, a, &p[0], &p[1], &p[2]);
    detector(G, b, &p[3], &p[4], &p[5]);
    p[0] = p[0] - ut * G->st[ka];
    p[1] = p[1] + ut * G->ct[ka];
    p[2] = p[2] + v;
    p[3] = p[3] + ut * G->st[kb];
    p[4] = p[4] - ut * G->ct[kb];
    p[5] = p[5] + v;
}

/* parametric interval [amin, amax] of the segment inside one slab */
static int slab(double p1, double d, double lo, uint32_t n, double v, double* amin, double* amax) {
    const double hi = lo + (double)n * v;
    if (d != 0.0) {
        const double a0 = (lo - p1) / d, an = (hi - p1) / d;
        *amin = fmax(*amin, fmin(a0, an));
        *amax = fmin(*amax, fmax(a0, an));
        return 1;
    }
    return p1 > lo && p1 < hi;
}

typedef struct {
    double next;
    int64_t plane;
    int dir;
} Crossing;

static Crossing first_crossing(double p1, double d, double lo, double v, double amin) {
    Crossing w;
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

static inline void next_crossing(Crossing* w, double p1, double d, double lo, double v) {
    w->plane += w->dir;
    w->next = (lo + (double)w->plane * v - p1) / d;
}

static inline int64_t clamp_index(int64_t v, int64_t n) { return v < 0 ? 0 : (v >= n ? n - 1 : v); }

typedef struct {
    uint64_t key; /* column << 5 | sub-ray */
    double len;
} Piece;

/* Traces one sub-ray; appends its (key, length) pieces to out; returns the count. */
static uint32_t trace(const Scan* G, const double p[6], uint32_t k, Piece* out) {
    const double p1x = p[0], p1y = p[1], p1z = p[2];
    const double dx = p[3] - p1x, dy = p[4] - p1y, dz = p[5] - p1z;
    const double L = sqrt(dx * dx + dy * dy + dz * dz);
    double amin = 0.0, amax = 1.0;
    if (!slab(p1x, dx, G->x0, G->nx, G->vx, &amin, &amax)) return 0;
    if (!slab(p1y, dy, G->y0, G->ny, G->vy, &amin, &amax)) return 0;
    if (!slab(p1z, dz, G->z0, G->nz, G->vz, &amin, &amax)) return 0;
    if (!(amax > amin)) return 0;
    Crossing wx = first_crossing(p1x, dx, G->x0, G->vx, amin);
    Crossing wy = first_crossing(p1y, dy, G->y0, G->vy, amin);
    Crossing wz = first_crossing(p1z, dz, G->z0, G->vz, amin);
    double acur = amin;
    uint32_t n = 0;
    uint32_t held_col = 0xffffffffu;
    double held_len = 0.0;
    const uint32_t guard = G->nx + G->ny + G->nz + 8;
    for (uint32_t it = 0; it < 2 * guard && acur < amax; ++it) {
        const double an = fmin(fmin(wx.next, wy.next), fmin(wz.next, amax));
        if (an > acur) {
            const double am = 0.5 * (acur + an);
            const int64_t ix = clamp_index((int64_t)floor((p1x + am * dx - G->x0) / G->vx), G->nx);
            const int64_t iy = clamp_index((int64_t)floor((p1y + am * dy - G->y0) / G->vy), G->ny);
            const int64_t iz = clamp_index((int64_t)floor((p1z + am * dz - G->z0) / G->vz), G->nz);
            const uint32_t c = (uint32_t)(ix + (int64_t)G->nx * (iy + (int64_t)G->ny * iz));
            const double len = (an - acur) * L;
            if (c == held_col) {
                held_len += len;
            } else {
                if (held_col != 0xffffffffu && held_len > kMinLen && n < G->cap_ray) {
                    out[n].key = ((uint64_t)held_col << 5) | k;
                    out[n].len = held_len;
                    ++n;
                }
                held_col = c;
                held_len = len;
            }
        }
        acur = an;
        if (wx.dir && wx.next <= an) next_crossing(&wx, p1x, dx, G->x0, G->vx);
        if (wy.dir && wy.next <= an) next_crossing(&wy, p1y, dy, G->y0, G->vy);
        if (wz.dir && wz.next <= an) next_crossing(&wz, p1z, dz, G->z0, G->vz);
    }
    if (held_col != 0xffffffffu && held_len > kMinLen && n < G->cap_ray) {
        out[n].key = ((uint64_t)held_col << 5) | k;
        out[n].len = held_len;
        ++n;
    }
    return n;
}

/* stable bottom-up merge sort of n pieces by key (tmp holds n pieces) */
static void sort_pieces(Piece* a, Piece* tmp, uint32_t n) {
    /* insertion sort of runs of 16, then merges */
    const uint32_t R = 16;
    for (uint32_t s = 0; s < n; s += R) {
        const uint32_t e = s + R < n ? s + R : n;
        for (uint32_t i = s + 1; i < e; ++i) {
            const Piece x = a[i];
            uint32_t j = i;
            while (j > s && a[j - 1].key > x.key) {
                a[j] = a[j - 1];
                --j;
            }
            a[j] = x;
        }
    }
    Piece* src = a;
    Piece* dst = tmp;
    for (uint32_t w = R; w < n; w *= 2) {
        for (uint32_t s = 0; s < n; s += 2 * w) {
            const uint32_t m = s + w < n ? s + w : n, e = s + 2 * w < n ? s + 2 * w : n;
            uint32_t i = s, j = m, o = s;
            while (i < m && j < e) dst[o++] = (src[j].key < src[i].key) ? src[j++] : src[i++];
            while (i < m) dst[o++] = src[i++];
            while (j < e) dst[o++] = src[j++];
        }
        Piece* t = src;
        src = dst;
        dst = t;
    }
    if (src != a) memcpy(a, src, sizeof(Piece) * n);
}

/* Row q: the union of its sub-rays, equal columns summed in sub-ray order,
 * value = sum / S.  Writes col/val when given; returns the element count. */
static uint32_t make_row(const Scan* G, uint64_t q, Piece* buf, Piece* tmp, uint32_t* col, float* val) {
    uint32_t a, b;
    pair_of(q * G->stride + G->phase, G->D, &a, &b);
    uint32_t n = 0;
    for (uint32_t k = 0; k < G->S; ++k) {
        double p[6];
        subray(G, a, b, k, p);
        n += trace(G, p, k, buf + n);
    }
    sort_pieces(buf, tmp, n);
    uint32_t m = 0;
    for (uint32_t i = 0; i < n;) {
        const uint64_t c = buf[i].key >> 5;
        double sum = 0.0;
        uint32_t j = i;
        for (; j < n && (buf[j].key >> 5) == c; ++j) sum += buf[j].len;
        if (col) {
            col[m] = (uint32_t)c;
            val[m] = (float)(sum / (double)G->S);
        }
        ++m;
        i = j;
    }
    return m;
}

uint64_t oracle_siddon_rows(const oracle_geometry* g) {
    Scan G;
    return make_scan(g, &G) == 0 ? G.nrows : 0;
}

/* Row pointers u64[rows+1]; returns 0, or -1 for an invalid geometry. */
int oracle_siddon_count(const oracle_geometry* g, uint64_t* rowptr) {
    Scan G;
    if (make_scan(g, &G) != 0) return -1;
    double* tab = (double*)malloc(sizeof(double) * 2 * G.dpr);
    angles(&G, tab, tab + G.dpr);
    G.ct = tab;
    G.st = tab + G.dpr;
    rowptr[0] = 0;
#pragma omp parallel
    {
        Piece* buf = (Piece*)malloc(sizeof(Piece) * (size_t)G.S * G.cap_ray);
        Piece* tmp = (Piece*)malloc(sizeof(Piece) * (size_t)G.S * G.cap_ray);
#pragma omp for schedule(dynamic, 256)
        for (int64_t q = 0; q < (int64_t)G.nrows; ++q) rowptr[q + 1] = make_row(&G, (uint64_t)q, buf, tmp, NULL, NULL);
        free(buf);
        free(tmp);
    }
    for (uint64_t q = 0; q < G.nrows; ++q) rowptr[q + 1] += rowptr[q];
    free(tab);
    return 0;
}

/* Fills col/val of the rows given by rowptr; returns 0, or -1 for an invalid geometry. */
int oracle_siddon_fill(const oracle_geometry* g, const uint64_t* rowptr, uint32_t* col, float* val) {
    Scan G;
    if (make_scan(g, &G) != 0) return -1;
    double* tab = (double*)malloc(sizeof(double) * 2 * G.dpr);
    angles(&G, tab, tab + G.dpr);
    G.ct = tab;
    G.st = tab + G.dpr;
#pragma omp parallel
    {
        Piece* buf = (Piece*)malloc(sizeof(Piece) * (size_t)G.S * G.cap_ray);
        Piece* tmp = (Piece*)malloc(sizeof(Piece) * (size_t)G.S * G.cap_ray);
#pragma omp for schedule(dynamic, 256)
        for (int64_t q = 0; q < (int64_t)G.nrows; ++q)
            make_row(&G, (uint64_t)q, buf, tmp, col + rowptr[q], val + rowptr[q]);
        free(buf);
        free(tmp);
    }
    free(tab);
    return 0;
}
