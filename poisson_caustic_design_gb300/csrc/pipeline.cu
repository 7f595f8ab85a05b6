// pipeline.cu -- the per-iteration mesh/grid steps of Caustic_design on sm_103a.
//
// Reference: src/caustic_design.cpp:190-364, src/mesh.cpp, src/polygon_utils.cpp.
// All arithmetic is FP64 (the reference's type); mesh and grid state stay in
// device memory across iterations and reach the host only through the getters.
//
// Kernels (one thread per unit):
//   k_mesh_init        vertex     generate_structured_mesh        mesh.cpp:45-64
//   k_minmax / k_scale cell       scale_matrix_proportional       utils.cpp:88-129
//   k_target_areas     vertex     get_target_partitioned_areas    polygon_utils.cpp:311-389
//   k_areas_errors     vertex     dual-cell shoelace + errors     mesh.cpp:174-231,
//                                 polygon_utils.cpp:216-236,401-414, caustic_design.cpp:195-209
//   k_scatter_owner    triangle   point location (replaces the BVH of bvh.cpp)
//   k_raster_gather    sample     barycentric interpolation       mesh.cpp:234-345
//   k_inverse_gather   vertex     calculate_inverted_transport_map mesh.cpp:348-409
//   k_normals          vertex     calculate_refractive_normals_uniform mesh.cpp:677-722
//   k_step             vertex     gradient + bilinear sample + step_grid + max |dp|
//                                 utils.cpp:3-20, caustic_design.cpp:156-188,228-265, mesh.cpp:485-532
//   k_height_sample    vertex     bilinear h + min + set_source_heights
//                                 caustic_design.cpp:320-331, mesh.cpp:724-742
//
// Point location: every triangle tests the grid samples (or query vertices)
// inside its bounding box with the reference's barycentric formula and
// +-1e-12 acceptance (bvh.cpp:162-217), and a sample keeps the lowest triangle
// index that accepts it (atomicMin), so the result does not depend on thread
// timing.  The reference keeps the first hit of its BVH walk instead; the two
// differ only for samples on shared edges, where the interpolants agree to
// rounding.
#include <climits>
#include <math_constants.h>
#include <cmath>
#include <cstring>
#include <vector>

#include "api_internal.cuh"
#include "design.cuh"

namespace pcd {

namespace {
constexpr int kT = 256;
constexpr double kSampleEps = 1e-8;   // mesh.cpp:241,298,351

inline int nblocks(long n, int cap = 1 << 20) { return (int)std::max<long>(1, std::min<long>(cap, (n + kT - 1) / kT)); }

__device__ __forceinline__ bool last_block_of(unsigned int *counter)
{
    __shared__ bool last;
    __syncthreads();
    if (threadIdx.x == 0) {
        __threadfence();
        last = atomicAdd(counter, 1u) == gridDim.x - 1;
    }
    __syncthreads();
    if (last) __threadfence();
    return last;
}

// Triangle t of the structured mesh (mesh.cpp:56-63): cell c = t/2 at
// (i, j) = (c / (nx-1), c % (nx-1)), v = i*nx + j;  even t: (v, v+1, v+nx),
// odd t: (v+nx, v+1, v+nx+1).
__device__ __forceinline__ void tri_vertices(int t, int nx, int v[3])
{
    const int c = t >> 1, i = c / (nx - 1), j = c - i * (nx - 1), base = i * nx + j;
    if ((t & 1) == 0) { v[0] = base; v[1] = base + 1; v[2] = base + nx; }
    else { v[0] = base + nx; v[1] = base + 1; v[2] = base + nx + 1; }
}

// Barycentric coordinates exactly as bvh.cpp:162-190 computes them for the
// triangle passed as (tri[2], tri[1], tri[0]); bc[k] weights vertex k.
// Returns the acceptance test of bvh.cpp:208-217.  Split into the triangle's
// part (edge vectors, Gram entries, the reciprocal of the determinant), done
// once per triangle, and the point's part: the same operations in the same
// order as one call, so the same bits.
struct BaryPre {
    double cx, cy, v0x, v0y, v1x, v1y, d00, d01, d11, inv;
};

__device__ __forceinline__ BaryPre bary_pre(double2 A, double2 B, double2 Cc)
{
    BaryPre t;
    t.cx = Cc.x;
    t.cy = Cc.y;
    t.v0x = A.x - Cc.x;
    t.v0y = A.y - Cc.y;
    t.v1x = B.x - Cc.x;
    t.v1y = B.y - Cc.y;
    t.d00 = __dadd_rn(__dmul_rn(t.v0x, t.v0x), __dmul_rn(t.v0y, t.v0y));
    t.d01 = __dadd_rn(__dmul_rn(t.v0x, t.v1x), __dmul_rn(t.v0y, t.v1y));
    t.d11 = __dadd_rn(__dmul_rn(t.v1x, t.v1x), __dmul_rn(t.v1y, t.v1y));
    const double denom = __dsub_rn(__dmul_rn(t.d00, t.d11), __dmul_rn(t.d01, t.d01));
    t.inv = 1.0 / denom;
    return t;
}

__device__ __forceinline__ bool bary_at(const BaryPre &t, double px, double py, double bc[3])
{
    const double v2x = px - t.cx, v2y = py - t.cy;
    const double d02 = __dadd_rn(__dmul_rn(t.v0x, v2x), __dmul_rn(t.v0y, v2y));
    const double d12 = __dadd_rn(__dmul_rn(t.v1x, v2x), __dmul_rn(t.v1y, v2y));
    const double u = __dmul_rn(__dsub_rn(__dmul_rn(t.d11, d02), __dmul_rn(t.d01, d12)), t.inv);
    const double v = __dmul_rn(__dsub_rn(__dmul_rn(t.d00, d12), __dmul_rn(t.d01, d02)), t.inv);
    const double eps = 1e-12;
    bc[0] = u;
    bc[1] = v;
    bc[2] = __dsub_rn(__dsub_rn(1.0, u), v);
    return (u >= -eps && v >= -eps) && (__dadd_rn(u, v) <= 1.0 + eps);
}

__device__ __forceinline__ bool bary(double2 A, double2 B, double2 Cc, double px, double py, double bc[3])
{
    return bary_at(bary_pre(A, B, Cc), px, py, bc);
}

__device__ __forceinline__ double sample_coord(int i, int n, double extent)
{
    // i*(extent-eps)/(n-1) + 0.5*eps   (mesh.cpp:245,252)
    return __dadd_rn(__ddiv_rn(__dmul_rn((double)i, extent - kSampleEps), (double)(n - 1)), 0.5 * kSampleEps);
}

__device__ __forceinline__ double2 source_xy(int k, int nx, int ny, double width, double height)
{
    const int i = k / nx, j = k - (k / nx) * nx;
    return make_double2(__ddiv_rn(__dmul_rn((double)j, width), (double)(nx - 1)),
                        __ddiv_rn(__dmul_rn((double)i, height), (double)(ny - 1)));
}

// ---------------------------------------------------------------------------
__global__ void k_mesh_init(double2 *tp, double *sz, int nx, int ny, double width, double height)
{
    const int n = nx * ny;
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) {
        tp[k] = source_xy(k, nx, ny, width, height);
        sz[k] = 0.0;
    }
}

// NaN-skipping min/max seeded with element 0 (utils.cpp:104-115).
__global__ void k_minmax(const double *g, long n, double *out, unsigned int *counter)
{
    double mn = g[0], mx = g[0];
    for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) {
        const double v = g[i];
        if (!isnan(v)) { mn = fmin(mn, v); mx = fmax(mx, v); }
    }
    mn = warp_min(mn);
    mx = -warp_min(-mx);
    __shared__ double smn[32], smx[32];
    if ((threadIdx.x & 31) == 0) { smn[threadIdx.x >> 5] = mn; smx[threadIdx.x >> 5] = mx; }
    __syncthreads();
    if (threadIdx.x < 32) {
        const int nw = blockDim.x >> 5;
        mn = threadIdx.x < nw ? smn[threadIdx.x] : mn;
        mx = threadIdx.x < nw ? smx[threadIdx.x] : mx;
        mn = warp_min(mn);
        mx = -warp_min(-mx);
        if (threadIdx.x == 0) { out[2 + 2 * blockIdx.x] = mn; out[3 + 2 * blockIdx.x] = mx; }
    }
    if (last_block_of(counter) && threadIdx.x == 0) {
        double a = out[2], b = out[3];
        for (int k = 1; k < (int)gridDim.x; k++) { a = fmin(a, out[2 + 2 * k]); b = fmax(b, out[3 + 2 * k]); }
        out[0] = a;
        out[1] = b;
        *counter = 0;
        __threadfence();
    }
}

// lo + (hi - lo) * (v - mn) / (mx - mn)   (utils.cpp:120-126); NaN stays 0.
__global__ void k_scale(const double *in, double *out, long n, const double *mm, double lo, double hi)
{
    const double mn = mm[0], mx = mm[1];
    for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) {
        const double v = in[i];
        out[i] = isnan(v) ? 0.0 : __dadd_rn(lo, __ddiv_rn(__dmul_rn(hi - lo, v - mn), mx - mn));
    }
}

// Up to six triangles around vertex (i, j) and the vertex's slot in each
// (the incidence of build_vertex_to_triangles, mesh.cpp:106-118).
__device__ __forceinline__ int vertex_triangles(int i, int j, int nx, int ny, int tri[6], int pos[6])
{
    int n = 0;
    const int cx = nx - 1;
    if (i < ny - 1 && j < nx - 1) { tri[n] = 2 * (i * cx + j); pos[n++] = 0; }
    if (i < ny - 1 && j > 0) {
        tri[n] = 2 * (i * cx + j - 1); pos[n++] = 1;
        tri[n] = 2 * (i * cx + j - 1) + 1; pos[n++] = 1;
    }
    if (i > 0 && j < nx - 1) {
        tri[n] = 2 * ((i - 1) * cx + j); pos[n++] = 2;
        tri[n] = 2 * ((i - 1) * cx + j) + 1; pos[n++] = 0;
    }
    if (i > 0 && j > 0) { tri[n] = 2 * ((i - 1) * cx + j - 1) + 1; pos[n++] = 2; }
    return n;
}

// Quad (v, mid(v,j), centroid(v,j,k), mid(v,k)) of get_triangle_quad
// (mesh.cpp:154-199) in coordinates relative to v, which keeps the shoelace
// sum free of the cancellation the absolute coordinates would cause.
__device__ __forceinline__ double quad_area_local(double2 a, double2 b, double2 c)
{
    const double bx = b.x - a.x, by = b.y - a.y, cx = c.x - a.x, cy = c.y - a.y;
    const double q1x = bx / 2.0, q1y = by / 2.0;
    const double q2x = (bx + cx) / 3.0, q2y = (by + cy) / 3.0;
    const double q3x = cx / 2.0, q3y = cy / 2.0;
    // shoelace over (0,0), q1, q2, q3; terms with the origin vanish
    return 0.5 * ((q1x * q2y - q2x * q1y) + (q2x * q3y - q3x * q2y));
}

__global__ void k_areas_errors(const double2 *__restrict__ tp, const double *__restrict__ target_areas,
                               double *__restrict__ areas, double *__restrict__ errors, int nx, int ny)
{
    const int n = nx * ny;
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) {
        const int i = k / nx, j = k - i * nx;
        int tri[6], pos[6];
        const int m = vertex_triangles(i, j, nx, ny, tri, pos);
        double a = 0.0;
        for (int q = 0; q < m; q++) {
            int v[3];
            tri_vertices(tri[q], nx, v);
            a += quad_area_local(tp[v[pos[q]]], tp[v[(pos[q] + 1) % 3]], tp[v[(pos[q] + 2) % 3]]);
        }
        areas[k] = a;
        // errors = (target - area) / area   (caustic_design.cpp:202-209)
        errors[k] = (target_areas[k] - a) / a;
    }
}

// ---- target areas (initialisation) ----------------------------------------
// Clip a convex polygon against s*(coord[axis] - c) >= 0.  Not inlined: its
// four call sites per pixel, each with the FP64 division's code, made the
// kernel wait on instruction fetch (no_instruction the first stall at 81 per
// issue); one shared copy runs the initialisation 22% faster.
__device__ __noinline__ int clip_half(const double2 *in, int n, double2 *out, int axis, double c, double s)
{
    int m = 0;
    for (int k = 0; k < n; k++) {
        const double2 p = in[k], q = in[(k + 1) % n];
        const double pa = axis ? p.y : p.x, qa = axis ? q.y : q.x;
        const double dp = s * (pa - c), dq = s * (qa - c);
        if (dp >= 0) out[m++] = p;
        if ((dp > 0 && dq < 0) || (dp < 0 && dq > 0)) {
            const double t = dp / (dp - dq);
            double2 r = make_double2(p.x + t * (q.x - p.x), p.y + t * (q.y - p.y));
            if (axis) r.y = c; else r.x = c;
            out[m++] = r;
        }
    }
    return m;
}

__device__ double quad_intensity(const double *img, int iw, int ih, double width, const double2 q[4])
{
    double xmin = q[0].x, xmax = q[0].x, ymin = q[0].y, ymax = q[0].y;
    for (int k = 1; k < 4; k++) {
        xmin = fmin(xmin, q[k].x); xmax = fmax(xmax, q[k].x);
        ymin = fmin(ymin, q[k].y); ymax = fmax(ymax, q[k].y);
    }
    const double px = width / (double)iw;
    const int ylo = (int)fmax(floor(ymin / px), 0.0), yhi = (int)fmin(ceil(ymax / px), (double)ih);
    const int xlo = (int)fmax(floor(xmin / px), 0.0), xhi = (int)fmin(ceil(xmax / px), (double)iw);
    double acc = 0.0;
    for (int y = ylo; y < yhi; y++)
        for (int x = xlo; x < xhi; x++) {
            const double cx = ((double)x + 0.5) * px, cy = ((double)y + 0.5) * px;
            double2 a[12], b[12];
            int n = clip_half(q, 4, a, 0, cx - px / 2.0, 1.0);
            n = clip_half(a, n, b, 0, cx + px / 2.0, -1.0);
            n = clip_half(b, n, a, 1, cy - px / 2.0, 1.0);
            n = clip_half(a, n, b, 1, cy + px / 2.0, -1.0);
            if (n >= 3) {
                double s = 0.0;
                for (int k = 0; k < n; k++) {
                    const int f = (k + 1) % n;
                    s += b[k].x * b[f].y - b[f].x * b[k].y;
                }
                acc += 0.5 * s * img[(long)y * iw + x];
            }
        }
    return acc;
}

__global__ void k_target_areas(const double2 *__restrict__ tp, const double *__restrict__ img, int iw, int ih,
                               double width, int nx, int ny, double *__restrict__ out, double *partials,
                               unsigned int *counter)
{
    const int n = nx * ny;
    double acc = 0.0;
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) {
        const int i = k / nx, j = k - i * nx;
        int tri[6], pos[6];
        const int m = vertex_triangles(i, j, nx, ny, tri, pos);
        double a = 0.0;
        for (int q = 0; q < m; q++) {
            int v[3];
            tri_vertices(tri[q], nx, v);
            const double2 A = tp[v[pos[q]]], B = tp[v[(pos[q] + 1) % 3]], Cc = tp[v[(pos[q] + 2) % 3]];
            double2 quad[4];
            quad[0] = A;
            quad[1] = make_double2((A.x + B.x) / 2.0, (A.y + B.y) / 2.0);
            quad[2] = make_double2((A.x + B.x + Cc.x) / 3.0, (A.y + B.y + Cc.y) / 3.0);
            quad[3] = make_double2((A.x + Cc.x) / 2.0, (A.y + Cc.y) / 2.0);
            a += quad_intensity(img, iw, ih, width, quad);
        }
        out[k] = a;
        acc += a;
    }
    double v[1] = {acc};
    block_reduce<1, 0u>(v);
    if (threadIdx.x == 0) partials[blockIdx.x] = v[0];
    if (last_block_of(counter)) {
        double w[1] = {0.0};
        for (int k = threadIdx.x; k < (int)gridDim.x; k += blockDim.x) w[0] += partials[k];
        block_reduce<1, 0u>(w);
        if (threadIdx.x == 0) {
            partials[gridDim.x] = w[0];
            *counter = 0;
            __threadfence();
        }
    }
}

// target_areas *= width*height / sum   (polygon_utils.cpp:382-386)
__global__ void k_scale_areas(double *areas, int n, const double *total, double wh)
{
    const double s = wh / *total;
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) areas[k] *= s;
}

// ---- point location ---------------------------------------------------------
// mode 0: grid samples (x_i, y_j) of mesh.cpp:241-254 on an rx x ry grid;
// mode 1: shrunk source vertices eps + s*((w-2eps)/w) of mesh.cpp:356-360.
// Both are separable, x from the column and y from the row, so their
// coordinates (each with an FP64 division) are computed once per design into
// per-axis tables cx[qx], cy[qy] (k_query_coords) and looked up.
struct QueryGrid {
    int mode;
    int qx, qy;  // query grid extents
    int nx, ny;  // mesh resolution
    double width, height;
    const double *cx, *cy;  // the query coordinates of each column and row
};

__device__ __forceinline__ double2 query_point_direct(const QueryGrid &g, int ix, int iy)
{
    if (g.mode == 0) return make_double2(sample_coord(ix, g.qx, g.width), sample_coord(iy, g.qy, g.height));
    const double2 s = source_xy(iy * g.nx + ix, g.nx, g.ny, g.width, g.height);
    return make_double2(__dadd_rn(kSampleEps, __dmul_rn(s.x, __ddiv_rn(g.width - 2 * kSampleEps, g.width))),
                        __dadd_rn(kSampleEps, __dmul_rn(s.y, __ddiv_rn(g.height - 2 * kSampleEps, g.height))));
}

__device__ __forceinline__ double2 query_point(const QueryGrid &g, int ix, int iy)
{
    return make_double2(__ldg(g.cx + ix), __ldg(g.cy + iy));
}

// The coordinate tables of a query grid: column ix's x from row 0, row iy's
// y from column 0 (the formulas above give every point of a column the same x).
__global__ void k_query_coords(QueryGrid g, double *cx, double *cy)
{
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < g.qx + g.qy; i += gridDim.x * blockDim.x) {
        if (i < g.qx) cx[i] = query_point_direct(g, i, 0).x;
        else cy[i - g.qx] = query_point_direct(g, 0, i - g.qx).y;
    }
}

__device__ __forceinline__ void query_range(const QueryGrid &g, double lo, double hi, int n, double extent, bool is_x,
                                            int &a, int &b)
{
    double fl, fh;
    if (g.mode == 0) {
        fl = (lo - 0.5 * kSampleEps) * (n - 1) / (extent - kSampleEps);
        fh = (hi - 0.5 * kSampleEps) * (n - 1) / (extent - kSampleEps);
    } else {
        const int m = is_x ? g.nx : g.ny;
        fl = lo * (m - 1) / extent;
        fh = hi * (m - 1) / extent;
    }
    a = (int)floor(fl) - 1;
    b = (int)ceil(fh) + 1;
    if (a < 0) a = 0;
    if (b > n - 1) b = n - 1;
}

__global__ void k_scatter_owner(const double2 *__restrict__ pts, QueryGrid g, unsigned int *__restrict__ owner)
{
    const int ntri = 2 * (g.nx - 1) * (g.ny - 1);
    for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < ntri; t += gridDim.x * blockDim.x) {
        int v[3];
        tri_vertices(t, g.nx, v);
        const double2 A = pts[v[0]], B = pts[v[1]], Cc = pts[v[2]];
        const double xmin = fmin(A.x, fmin(B.x, Cc.x)), xmax = fmax(A.x, fmax(B.x, Cc.x));
        const double ymin = fmin(A.y, fmin(B.y, Cc.y)), ymax = fmax(A.y, fmax(B.y, Cc.y));
        int ilo, ihi, jlo, jhi;
        query_range(g, xmin, xmax, g.qx, g.width, true, ilo, ihi);
        query_range(g, ymin, ymax, g.qy, g.height, false, jlo, jhi);
        const BaryPre pre = bary_pre(A, B, Cc);
        for (int jy = jlo; jy <= jhi; jy++) {
            const double py = __ldg(g.cy + jy);
            for (int ix = ilo; ix <= ihi; ix++) {
                const long s = (long)jy * g.qx + ix;
                if (owner[s] <= (unsigned)t) continue;  // a lower triangle already holds it
                double bc[3];
                if (bary_at(pre, __ldg(g.cx + ix), py, bc)) atomicMin(&owner[s], (unsigned)t);
            }
        }
    }
}

// Raster values: out_k[s] = sum_v vals_k[tri v] * bc_v  for up to two fields.
__global__ void k_raster_gather(const double2 *__restrict__ pts, QueryGrid g, const unsigned int *__restrict__ owner,
                                const double *__restrict__ va, const double *__restrict__ vb, double *__restrict__ oa,
                                double *__restrict__ ob, unsigned int *misses)
{
    const long n = (long)g.qx * g.qy;
    unsigned int miss = 0;
    for (long s = (long)blockIdx.x * blockDim.x + threadIdx.x; s < n; s += (long)gridDim.x * blockDim.x) {
        const unsigned int t = owner[s];
        if (t == UINT_MAX) {
            oa[s] = CUDART_NAN;
            if (ob) ob[s] = CUDART_NAN;
            miss++;
            continue;
        }
        int v[3];
        tri_vertices((int)t, g.nx, v);
        const int iy = (int)(s / g.qx), ix = (int)(s - (long)iy * g.qx);
        const double2 p = query_point(g, ix, iy);
        double bc[3];
        bary(pts[v[0]], pts[v[1]], pts[v[2]], p.x, p.y, bc);
        // interpolation = v0*b0 + v1*b1 + v2*b2   (mesh.cpp:270-273)
        oa[s] = __dadd_rn(__dadd_rn(__dmul_rn(va[v[0]], bc[0]), __dmul_rn(va[v[1]], bc[1])), __dmul_rn(va[v[2]], bc[2]));
        if (ob)
            ob[s] = __dadd_rn(__dadd_rn(__dmul_rn(vb[v[0]], bc[0]), __dmul_rn(vb[v[1]], bc[1])),
                              __dmul_rn(vb[v[2]], bc[2]));
    }
    if (miss) atomicAdd(misses, miss);
}

// Inverse transport map: interpolate the (uniform) source positions at each
// located source vertex and pin boundary vertices (mesh.cpp:365-402).
__global__ void k_inverse_gather(const double2 *__restrict__ tp, QueryGrid g, const unsigned int *__restrict__ owner,
                                 double2 *__restrict__ inv, unsigned int *misses)
{
    const int n = g.nx * g.ny;
    unsigned int miss = 0;
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) {
        const unsigned int t = owner[k];
        if (t == UINT_MAX) {
            inv[k] = make_double2(CUDART_NAN, CUDART_NAN);
            miss++;
            continue;
        }
        int v[3];
        tri_vertices((int)t, g.nx, v);
        const int i = k / g.nx, j = k - i * g.nx;
        const double2 p = query_point(g, j, i);
        double bc[3];
        bary(tp[v[0]], tp[v[1]], tp[v[2]], p.x, p.y, bc);
        const double2 s0 = source_xy(v[0], g.nx, g.ny, g.width, g.height);
        const double2 s1 = source_xy(v[1], g.nx, g.ny, g.width, g.height);
        const double2 s2 = source_xy(v[2], g.nx, g.ny, g.width, g.height);
        const double ix = __dadd_rn(__dadd_rn(__dmul_rn(s0.x, bc[0]), __dmul_rn(s1.x, bc[1])), __dmul_rn(s2.x, bc[2]));
        const double iy = __dadd_rn(__dadd_rn(__dmul_rn(s0.y, bc[0]), __dmul_rn(s1.y, bc[1])), __dmul_rn(s2.y, bc[2]));
        const double ox = (j == 0) ? 0.0 : (j == g.nx - 1 ? g.width : ix);
        const double oy = (i == 0) ? 0.0 : (i == g.ny - 1 ? g.height : iy);
        inv[k] = make_double2(ox, oy);
    }
    if (miss) atomicAdd(misses, miss);
}

// Refractive surface slopes (mesh.cpp:695-719): t = normalize(inv - s_xy,
// f - s_z); n = t - ri*(0,0,1); output (n_x/n_z, n_y/n_z).
__global__ void k_normals(const double2 *__restrict__ inv, const double *__restrict__ sz, int nx, int ny,
                          double width, double height, double focal, double ri, double *__restrict__ onx,
                          double *__restrict__ ony)
{
    const int n = nx * ny;
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) {
        const double2 s = source_xy(k, nx, ny, width, height);
        double t0 = inv[k].x - s.x, t1 = inv[k].y - s.y, t2 = 0.0 - sz[k] + focal;
        const double len = sqrt(__dadd_rn(__dadd_rn(__dmul_rn(t0, t0), __dmul_rn(t1, t1)), __dmul_rn(t2, t2)));
        t0 = t0 / len;
        t1 = t1 / len;
        t2 = t2 / len;
        const double zz = t2 - ri;
        onx[k] = t0 / zz;
        ony[k] = t1 / zz;
    }
}

// Bilinear sample with floor/ceil corners clamped to the grid
// (caustic_design.cpp:156-188).  G(x, y) supplies grid values.
template <typename G>
__device__ __forceinline__ double bilinear(const G &grid, int W, int H, double x, double y)
{
    int x0 = (int)floor(x), y0 = (int)floor(y), x1 = (int)ceil(x), y1 = (int)ceil(y);
    x0 = min(max(x0, 0), W - 1);
    x1 = min(max(x1, 0), W - 1);
    y0 = min(max(y0, 0), H - 1);
    y1 = min(max(y1, 0), H - 1);
    const double fx1 = x - x0, fx0 = 1.0 - fx1;
    const double fy1 = y - y0, fy0 = 1.0 - fy1;
    const double top = __dadd_rn(__dmul_rn(fx0, grid(x0, y0)), __dmul_rn(fx1, grid(x1, y0)));
    const double bot = __dadd_rn(__dmul_rn(fx0, grid(x0, y1)), __dmul_rn(fx1, grid(x1, y1)));
    return __dadd_rn(__dmul_rn(fy0, top), __dmul_rn(fy1, bot));
}

struct GradX {
    const double *phi;
    int W, H;
    __device__ double operator()(int x, int y) const
    {
        return (phi[(long)y * W + min(x + 1, W - 1)] - phi[(long)y * W + max(x - 1, 0)]) / 2.0;
    }
};
struct GradY {
    const double *phi;
    int W, H;
    __device__ double operator()(int x, int y) const
    {
        return (phi[(long)min(y + 1, H - 1) * W + x] - phi[(long)max(y - 1, 0) * W + x]) / 2.0;
    }
};
struct Plain {
    const double *g;
    int W;
    __device__ double operator()(int x, int y) const { return g[(long)y * W + x]; }
};

// Vertex step: gradient of phi sampled at ((x/width)*rx - 0.5, (y/height)*ry
// - 0.5), edge vertices slide along their edge, corners stay, p += v*dt*step
// with dt = width/nx; the largest |dp| goes to *maxbits.
__global__ void k_step(double2 *__restrict__ tp, const double *__restrict__ phi, int rx, int ry, int nx, int ny,
                       double width, double height, double step, double *__restrict__ vgx, double *__restrict__ vgy,
                       unsigned long long *maxbits)
{
    const int n = nx * ny;
    const GradX gxf{phi, rx, ry};
    const GradY gyf{phi, rx, ry};
    const double dt = width / nx;
    double best = 0.0;
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) {
        const double2 p = tp[k];
        const double sx = __dsub_rn(__dmul_rn(__ddiv_rn(p.x, width), (double)rx), 0.5);
        const double sy = __dsub_rn(__dmul_rn(__ddiv_rn(p.y, height), (double)ry), 0.5);
        const double gx = bilinear(gxf, rx, ry, sx, sy);
        const double gy = bilinear(gyf, rx, ry, sx, sy);
        vgx[k] = gx;
        vgy[k] = gy;
        const int i = k / nx, j = k - i * nx;
        const bool xedge = (j == 0 || j == nx - 1), yedge = (i == 0 || i == ny - 1);
        const double vx = xedge ? 0.0 : gx, vy = yedge ? 0.0 : gy;
        const double2 q = make_double2(__dadd_rn(p.x, __dmul_rn(__dmul_rn(vx, dt), step)),
                                       __dadd_rn(p.y, __dmul_rn(__dmul_rn(vy, dt), step)));
        tp[k] = q;
        const double dx = p.x - q.x, dy = p.y - q.y;
        const double d = sqrt(__dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy)));
        best = nan_skip_max(best, d);
    }
    best = warp_max(best);
    __shared__ double sm[32];
    if ((threadIdx.x & 31) == 0) sm[threadIdx.x >> 5] = best;
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int w = 1; w < (int)(blockDim.x >> 5); w++) best = nan_skip_max(best, sm[w]);
        if (best > 0.0) atomicMax(maxbits, (unsigned long long)__double_as_longlong(best));
    }
}

// Heights: hv = bilinear(h) at the source vertices (caustic_design.cpp:323-329).
__global__ void k_height_sample(const double *__restrict__ h, int rx, int ry, int nx, int ny, double width,
                                double height, double *__restrict__ hv, double *partials, unsigned int *counter)
{
    const int n = nx * ny;
    const Plain g{h, rx};
    double mn = 0.0;  // min(0, min hv)  (mesh.cpp:726-733)
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) {
        const double2 s = source_xy(k, nx, ny, width, height);
        const double sx = __dsub_rn(__dmul_rn(__ddiv_rn(s.x, width), (double)rx), 0.5);
        const double sy = __dsub_rn(__dmul_rn(__ddiv_rn(s.y, height), (double)ry), 0.5);
        const double v = bilinear(g, rx, ry, sx, sy);
        hv[k] = v;
        if (mn > v) mn = v;
    }
    mn = warp_min(mn);
    __shared__ double sm[32];
    if ((threadIdx.x & 31) == 0) sm[threadIdx.x >> 5] = mn;
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int w = 1; w < (int)(blockDim.x >> 5); w++) mn = fmin(mn, sm[w]);
        partials[1 + blockIdx.x] = mn;
    }
    if (last_block_of(counter) && threadIdx.x == 0) {
        double m = 0.0;
        for (int b = 0; b < (int)gridDim.x; b++) m = fmin(m, partials[1 + b]);
        partials[0] = m;
        *counter = 0;
        __threadfence();
    }
}

// z = hv - m; sum (z_new - z_old)^2  (mesh.cpp:735-741), deterministic sum.
__global__ void k_height_apply(const double *__restrict__ hv, double *__restrict__ sz, int n, double *partials,
                               unsigned int *counter, double *out_sum)
{
    const double m = partials[0];
    double acc = 0.0;
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) {
        const double v = hv[k] - m;
        const double d = v - sz[k];
        acc += d * d;
        sz[k] = v;
    }
    double w[1] = {acc};
    block_reduce<1, 0u>(w);
    if (threadIdx.x == 0) partials[1 + blockIdx.x] = w[0];
    if (last_block_of(counter)) {
        double u[1] = {0.0};
        for (int b = threadIdx.x; b < (int)gridDim.x; b += blockDim.x) u[0] += partials[1 + b];
        block_reduce<1, 0u>(u);
        if (threadIdx.x == 0) {
            *out_sum = u[0];
            *counter = 0;
            __threadfence();
        }
    }
}

__global__ void k_points_out(const double2 *xy, const double *z, int nx, int ny, double width, double height,
                             int source, double *out)
{
    const int n = nx * ny;
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) {
        const double2 p = source ? source_xy(k, nx, ny, width, height) : xy[k];
        out[3L * k] = p.x;
        out[3L * k + 1] = p.y;
        out[3L * k + 2] = source ? z[k] : 0.0;
    }
}

// Mesh::laplacian_smoothing mesh.cpp:534-606, pass 1: the neighbour means
// (same summation order as the reference) into `mean`.
__global__ void k_smooth_mean(const double2 *__restrict__ tp, int nx, int ny, double2 *__restrict__ mean)
{
    const int n = nx * ny;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const int y = i / nx, x = i - y * nx;
        double2 q = tp[i];
        const bool corner = (x == 0 || x == nx - 1) && (y == 0 || y == ny - 1);
        if (corner) {
        } else if (x == 0) {
            q.y = ((0.0 + tp[i + 1].y) + tp[i + nx].y) + tp[i - nx].y;
            q.y /= 3.0;
        } else if (x == nx - 1) {
            q.y = ((0.0 + tp[i - 1].y) + tp[i - nx].y) + tp[i + nx].y;
            q.y /= 3.0;
        } else if (y == 0) {
            q.x = ((0.0 + tp[i - 1].x) + tp[i + 1].x) + tp[i + nx].x;
            q.x /= 3.0;
        } else if (y == ny - 1) {
            q.x = ((0.0 + tp[i - 1].x) + tp[i - nx].x) + tp[i + 1].x;
            q.x /= 3.0;
        } else {
            q.x = (((0.0 + tp[i - 1].x) + tp[i + 1].x) + tp[i - nx].x) + tp[i + nx].x;
            q.y = (((0.0 + tp[i - 1].y) + tp[i + 1].y) + tp[i - nx].y) + tp[i + nx].y;
            q.x /= 4.0;
            q.y /= 4.0;
        }
        mean[i] = q;
    }
}

// pass 2: p = mean * f + p * (1 - f)
__global__ void k_smooth_apply(double2 *__restrict__ tp, const double2 *__restrict__ mean, int n, double f)
{
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const double2 m = mean[i], p = tp[i];
        tp[i] = make_double2(__dadd_rn(__dmul_rn(m.x, f), __dmul_rn(p.x, 1.0 - f)),
                             __dadd_rn(__dmul_rn(m.y, f), __dmul_rn(p.y, 1.0 - f)));
    }
}

// triangles {i, i+1, i+nx}, {i+nx, i+1, i+nx+1} (mesh.cpp:57-63) with signed area <= 0
__global__ void k_count_folds(const double2 *__restrict__ tp, int nx, int ny, unsigned long long *count)
{
    unsigned long long local = 0;
    const long nq = (long)(nx - 1) * (ny - 1);
    for (long q = (long)blockIdx.x * blockDim.x + threadIdx.x; q < nq; q += (long)gridDim.x * blockDim.x) {
        const int y = (int)(q / (nx - 1)), x = (int)(q - (long)y * (nx - 1));
        const long i = (long)y * nx + x;
        const long t[2][3] = {{i, i + 1, i + nx}, {i + nx, i + 1, i + nx + 1}};
        for (int k = 0; k < 2; k++) {
            const double2 a = tp[t[k][0]], b = tp[t[k][1]], c = tp[t[k][2]];
            const double area2 = __dsub_rn(__dmul_rn(b.x - a.x, c.y - a.y), __dmul_rn(c.x - a.x, b.y - a.y));
            if (!(area2 > 0.0)) local++;
        }
    }
    for (int o = 16; o > 0; o >>= 1) local += __shfl_xor_sync(0xffffffffu, local, o);
    if ((threadIdx.x & 31) == 0 && local) atomicAdd(count, local);
}

// The query grid of a design: mode 0 its rx x ry raster samples, mode 1 its
// shrunk source vertices, with the coordinate tables filled at initialisation
// (qc: rx sample x, ry sample y, nx source x, ny source y).
QueryGrid query_grid(const Design &d, int mode)
{
    const pcd_design_params &p = d.p;
    QueryGrid g{mode, mode ? p.mesh_res_x : p.res_x, mode ? p.mesh_res_y : p.res_y, p.mesh_res_x, p.mesh_res_y,
                p.width, p.height, nullptr, nullptr};
    g.cx = mode ? d.qc + p.res_x + p.res_y : d.qc;
    g.cy = g.cx + g.qx;
    return g;
}

}  // namespace

// ---------------------------------------------------------------------------
int Design::alloc()
{
    const size_t nv = (size_t)p.mesh_res_x * p.mesh_res_y;
    const size_t ng = (size_t)p.res_x * p.res_y;
    const size_t nq = std::max(ng, nv);
    PCD_CUDA(cudaMalloc(&tp, nv * sizeof(double2)));
    PCD_CUDA(cudaMalloc(&src_xy, nv * sizeof(double2)));
    PCD_CUDA(cudaMalloc(&inv, nv * sizeof(double2)));
    PCD_CUDA(cudaMalloc(&tp_cells, nv * sizeof(double2)));
    PCD_CUDA(cudaMalloc(&pts_out, 3 * nv * sizeof(double)));
    double **vbufs[] = {&sz, &target_areas, &areas, &errors, &vgx, &vgy, &nrm_x, &nrm_y, &hv};
    for (double **b : vbufs) PCD_CUDA(cudaMalloc(b, nv * sizeof(double)));
    double **gbufs[] = {&pixels, &raster, &phi, &h, &norm_x, &norm_y, &div};
    for (double **b : gbufs) PCD_CUDA(cudaMalloc(b, ng * sizeof(double)));
    PCD_CUDA(cudaMalloc(&owner, nq * sizeof(unsigned int)));
    PCD_CUDA(cudaMalloc(&qc, sizeof(double) * ((size_t)p.res_x + p.res_y + p.mesh_res_x + p.mesh_res_y)));
    PCD_CUDA(cudaMalloc(&scratch, sizeof(double) * (4 + 2 * 4096)));
    PCD_CUDA(cudaMalloc(&counter, 4 * sizeof(unsigned int)));
    PCD_CUDA(cudaMemset(counter, 0, 4 * sizeof(unsigned int)));
    PCD_CUDA(cudaMalloc(&small, 8 * sizeof(unsigned long long)));
    PCD_CUDA(cudaMallocHost(&small_host, 8 * sizeof(unsigned long long)));
    return PCD_OK;
}

void Design::release()
{
    void *bufs[] = {tp, src_xy, pts_out, inv, tp_cells, grad, sz, target_areas, areas, errors, vgx, vgy, nrm_x, nrm_y, hv, pixels, raster,
                    phi, h, norm_x, norm_y, div, owner, scratch, counter, small, qc};
    for (void *b : bufs)
        if (b) cudaFree(b);
    if (small_host) cudaFreeHost(small_host);
    tp = src_xy = inv = tp_cells = nullptr;
    grad = nullptr;
    pts_out = sz = target_areas = areas = errors = vgx = vgy = nrm_x = nrm_y = hv = nullptr;
    pixels = raster = phi = h = norm_x = norm_y = div = nullptr;
    owner = counter = nullptr;
    scratch = qc = nullptr;
    small = small_host = nullptr;
    initialized = false;
}

int Design::locate(const double2 *pts, int mode, int qx, int qy, cudaStream_t s)
{
    const QueryGrid g = query_grid(*this, mode);
    PCD_CUDA(cudaMemsetAsync(owner, 0xFF, sizeof(unsigned int) * (size_t)qx * qy, s));
    const int ntri = 2 * (p.mesh_res_x - 1) * (p.mesh_res_y - 1);
    k_scatter_owner<<<nblocks(ntri), kT, 0, s>>>(pts, g, owner);
    PCD_LAUNCHED(1);
    return PCD_OK;
}

int Design::raster_values(const double2 *pts, const double *va, const double *vb, double *oa, double *ob,
                          cudaStream_t s, unsigned int *misses_host)
{
    const int rx = p.res_x, ry = p.res_y;
    PCD_TRY(locate(pts, 0, rx, ry, s));
    const QueryGrid g = query_grid(*this, 0);
    unsigned int *miss = (unsigned int *)small;
    PCD_CUDA(cudaMemsetAsync(miss, 0, sizeof(unsigned int), s));
    k_raster_gather<<<nblocks((long)rx * ry, 4096), kT, 0, s>>>(pts, g, owner, va, vb, oa, ob, miss);
    PCD_LAUNCHED(1);
    PCD_CUDA(cudaMemcpyAsync(small_host, miss, sizeof(unsigned int), cudaMemcpyDeviceToHost, s));
    PCD_CUDA(cudaStreamSynchronize(s));
    *misses_host = *(unsigned int *)small_host;
    return PCD_OK;
}

int Design::initialize(const double *image_host)
{
    cudaStream_t s = ctx->stream;
    const int nx = p.mesh_res_x, ny = p.mesh_res_y, rx = p.res_x, ry = p.res_y;
    const long ng = (long)rx * ry;
    const int nv = nx * ny;
    // pixels = scale_matrix_proportional(image, 0, 1)   (caustic_design.cpp:335)
    PCD_CUDA(cudaMemcpyAsync(raster, image_host, ng * sizeof(double), cudaMemcpyHostToDevice, s));
    const int gb = nblocks(ng, 1024);
    k_minmax<<<gb, kT, 0, s>>>(raster, ng, scratch, counter);
    PCD_LAUNCHED(1);
    k_scale<<<gb, kT, 0, s>>>(raster, pixels, ng, scratch, 0.0, 1.0);
    PCD_LAUNCHED(1);
    // mesh (caustic_design.cpp:339)
    k_mesh_init<<<nblocks(nv), kT, 0, s>>>(tp, sz, nx, ny, p.width, p.height);
    PCD_LAUNCHED(1);
    PCD_CUDA(cudaMemcpyAsync(src_xy, tp, nv * sizeof(double2), cudaMemcpyDeviceToDevice, s));
    PCD_CUDA(cudaMemcpyAsync(tp_cells, tp, nv * sizeof(double2), cudaMemcpyDeviceToDevice, s));
    // coordinate tables of the two query grids (raster samples, source vertices)
    for (int mode = 0; mode < 2; mode++) {
        const QueryGrid g = query_grid(*this, mode);
        k_query_coords<<<nblocks(g.qx + g.qy), kT, 0, s>>>(g, const_cast<double *>(g.cx), const_cast<double *>(g.cy));
        PCD_LAUNCHED(1);
    }
    // target areas (caustic_design.cpp:348)
    const int vb = nblocks(nv, 2048);
    k_target_areas<<<vb, kT, 0, s>>>(tp, pixels, rx, ry, p.width, nx, ny, target_areas, scratch, counter);
    PCD_LAUNCHED(1);
    k_scale_areas<<<nblocks(nv), kT, 0, s>>>(target_areas, nv, scratch + vb, p.width * p.height);
    PCD_LAUNCHED(1);
    // phi = h = 0 (caustic_design.cpp:354-363)
    PCD_CUDA(cudaMemsetAsync(phi, 0, ng * sizeof(double), s));
    PCD_CUDA(cudaMemsetAsync(h, 0, ng * sizeof(double), s));
    PCD_CUDA(cudaMemsetAsync(raster, 0, ng * sizeof(double), s));
    PCD_CUDA(cudaStreamSynchronize(s));
    initialized = true;
    return PCD_OK;
}

int Design::transport_pre(double *step_out)
{
    if (!initialized) {
        set_error("pcd_design_transport_iteration: initialize first");
        return PCD_BAD_ARG;
    }
    cudaStream_t s = ctx->stream;
    const int nx = p.mesh_res_x, ny = p.mesh_res_y, rx = p.res_x, ry = p.res_y;
    const int nv = nx * ny;
    // the mesh the dual cells are built from (target_cells, caustic_design.cpp:195-196)
    PCD_CUDA(cudaMemcpyAsync(tp_cells, tp, nv * sizeof(double2), cudaMemcpyDeviceToDevice, s));
    // dual-cell areas and errors (caustic_design.cpp:195-209)
    k_areas_errors<<<nblocks(nv), kT, 0, s>>>(tp, target_areas, areas, errors, nx, ny);
    PCD_LAUNCHED(1);
    // rasterise the errors on the deformed mesh (caustic_design.cpp:213)
    unsigned int misses = 0;
    PCD_TRY(raster_values(tp, errors, nullptr, raster, nullptr, s, &misses));
    if (misses) {
        if (step_out) *step_out = NAN;
        if (p.raster_miss_policy == 1) {
            // caustic_design.cpp:214-217 (unreached in the reference, which
            // exits first): smooth the target mesh with the float literal 0.1f
            PCD_TRY(smooth_target((double)0.1f));
            return PCD_MESH_SMOOTHED;
        }
        set_error("raster miss: " + std::to_string(misses) + " grid samples outside every triangle");
        return PCD_RASTER_MISS;
    }
    // subtractAverage (caustic_design.cpp:221); the solve of raster into phi follows
    PCD_TRY(subtract_average(ctx->grid, raster, (long)rx * ry, s));
    return PCD_OK;
}

int Design::transport_post(double *step_out)
{
    cudaStream_t s = ctx->stream;
    const int nx = p.mesh_res_x, ny = p.mesh_res_y, rx = p.res_x, ry = p.res_y;
    const int nv = nx * ny;
    // gradient, vertex sampling, step_grid, max displacement (caustic_design.cpp:225-265)
    unsigned long long *maxbits = small + 1;
    PCD_CUDA(cudaMemsetAsync(maxbits, 0, sizeof(unsigned long long), s));
    const double step = (double)0.05f;  // the float literal of caustic_design.cpp:250
    k_step<<<nblocks(nv), kT, 0, s>>>(tp, phi, rx, ry, nx, ny, p.width, p.height, step, vgx, vgy, maxbits);
    PCD_LAUNCHED(1);
    PCD_CUDA(cudaMemcpyAsync(small_host + 1, maxbits, sizeof(unsigned long long), cudaMemcpyDeviceToHost, s));
    PCD_CUDA(cudaStreamSynchronize(s));
    double mx;
    std::memcpy(&mx, small_host + 1, sizeof(double));
    if (step_out) *step_out = mx / p.width;
    return PCD_OK;
}

int Design::transport_iteration(double *step_out, pcd_solve_stats *stats)
{
    const int pre = transport_pre(step_out);
    if (pre != PCD_OK) return pre;
    // poisson_solver (caustic_design.cpp:222)
    pcd_solve_stats st{};
    int ss = solve_device(ctx->solver, raster, phi, p.res_x, p.res_y, p.res_x, p.transport, &st, ctx->stream);
    if (ss != PCD_OK && ss != PCD_NOT_CONVERGED) return ss;
    if (stats) *stats = st;
    return transport_post(step_out);
}

int Design::height_pre()
{
    if (!initialized) {
        set_error("pcd_design_height_iteration: initialize first");
        return PCD_BAD_ARG;
    }
    cudaStream_t s = ctx->stream;
    const int nx = p.mesh_res_x, ny = p.mesh_res_y, rx = p.res_x, ry = p.res_y;
    const int nv = nx * ny;
    // inverse transport map (mesh.cpp:348-409)
    PCD_TRY(locate(tp, 1, nx, ny, s));
    const QueryGrid g = query_grid(*this, 1);
    unsigned int *miss = (unsigned int *)small;
    PCD_CUDA(cudaMemsetAsync(miss, 0, sizeof(unsigned int), s));
    k_inverse_gather<<<nblocks(nv), kT, 0, s>>>(tp, g, owner, inv, miss);
    PCD_LAUNCHED(1);
    // normals with focal length in grid units (caustic_design.cpp:271)
    const double focal = p.res_x / p.width * p.focal_l;
    k_normals<<<nblocks(nv), kT, 0, s>>>(inv, sz, nx, ny, p.width, p.height, focal, 1.49, nrm_x, nrm_y);
    PCD_LAUNCHED(1);
    PCD_CUDA(cudaMemcpyAsync(small_host, miss, sizeof(unsigned int), cudaMemcpyDeviceToHost, s));
    PCD_CUDA(cudaStreamSynchronize(s));
    if (*(unsigned int *)small_host) {
        set_error("inverse map miss: a source vertex lies in no deformed triangle");
        return PCD_RASTER_MISS;
    }
    // source-mesh raster of both slopes (caustic_design.cpp:274-277); the
    // source positions are the undeformed uniform grid
    unsigned int misses = 0;
    PCD_TRY(raster_values(src_xy, nrm_x, nrm_y, norm_x, norm_y, s, &misses));
    if (misses) {
        set_error("raster miss on the source mesh");
        return PCD_RASTER_MISS;
    }
    // divergence + subtractAverage (caustic_design.cpp:307-310); the solve of
    // div into h follows
    PCD_TRY(divergence(norm_x, norm_y, div, rx, ry, s));
    PCD_TRY(subtract_average(ctx->grid, div, (long)rx * ry, s));
    return PCD_OK;
}

int Design::height_post(double *update_out)
{
    cudaStream_t s = ctx->stream;
    const int nx = p.mesh_res_x, ny = p.mesh_res_y, rx = p.res_x, ry = p.res_y;
    const int nv = nx * ny;
    // heights (caustic_design.cpp:323-330)
    const int vb = nblocks(nv, 2048);
    k_height_sample<<<vb, kT, 0, s>>>(h, rx, ry, nx, ny, p.width, p.height, hv, scratch, counter);
    PCD_LAUNCHED(1);
    double *sum = scratch + 4096 + 8;
    k_height_apply<<<vb, kT, 0, s>>>(hv, sz, nv, scratch, counter + 1, sum);
    PCD_LAUNCHED(1);
    PCD_CUDA(cudaMemcpyAsync(small_host + 2, sum, sizeof(double), cudaMemcpyDeviceToHost, s));
    PCD_CUDA(cudaStreamSynchronize(s));
    double u;
    std::memcpy(&u, small_host + 2, sizeof(double));
    if (update_out) *update_out = u;
    return PCD_OK;
}

int Design::height_iteration(int itr, double *update_out, pcd_solve_stats *stats)
{
    (void)itr;
    PCD_TRY(height_pre());
    // poisson_solver on the divergence (caustic_design.cpp:311)
    pcd_solve_stats st{};
    int ss = solve_device(ctx->solver, div, h, p.res_x, p.res_y, p.res_x, p.height_solve, &st, ctx->stream);
    if (ss != PCD_OK && ss != PCD_NOT_CONVERGED) return ss;
    if (stats) *stats = st;
    return height_post(update_out);
}

int Design::smooth_target(double f)
{
    cudaStream_t s = ctx->stream;
    const int nx = p.mesh_res_x, ny = p.mesh_res_y, nv = nx * ny;
    k_smooth_mean<<<nblocks(nv), kT, 0, s>>>(tp, nx, ny, inv);  // inv: scratch, recomputed on use
    PCD_LAUNCHED(1);
    k_smooth_apply<<<nblocks(nv), kT, 0, s>>>(tp, inv, nv, f);
    PCD_LAUNCHED(1);
    PCD_CUDA(cudaStreamSynchronize(s));
    return PCD_OK;
}

int Design::count_folds(long long *folds)
{
    cudaStream_t s = ctx->stream;
    const int nx = p.mesh_res_x, ny = p.mesh_res_y;
    unsigned long long *cnt = small + 2;
    PCD_CUDA(cudaMemsetAsync(cnt, 0, sizeof(unsigned long long), s));
    k_count_folds<<<nblocks((long)(nx - 1) * (ny - 1)), kT, 0, s>>>(tp, nx, ny, cnt);
    PCD_LAUNCHED(1);
    PCD_CUDA(cudaMemcpyAsync(small_host + 3, cnt, sizeof(unsigned long long), cudaMemcpyDeviceToHost, s));
    PCD_CUDA(cudaStreamSynchronize(s));
    *folds = (long long)small_host[3];
    return PCD_OK;
}

int Design::set_target_points(const double *pts3)
{
    const int nv = p.mesh_res_x * p.mesh_res_y;
    std::vector<double2> h((size_t)nv);
    for (int i = 0; i < nv; i++) h[(size_t)i] = make_double2(pts3[3 * i], pts3[3 * i + 1]);
    PCD_CUDA(cudaMemcpyAsync(tp, h.data(), sizeof(double2) * nv, cudaMemcpyHostToDevice, ctx->stream));
    PCD_CUDA(cudaStreamSynchronize(ctx->stream));
    return PCD_OK;
}

int Design::get_grid(int which, double *out)
{
    const double *src = nullptr;
    switch (which) {
    case PCD_GRID_PHI: src = phi; break;
    case PCD_GRID_H: src = h; break;
    case PCD_GRID_RASTER: src = raster; break;
    case PCD_GRID_DIVERGENCE: src = div; break;
    case PCD_GRID_NORM_X: src = norm_x; break;
    case PCD_GRID_NORM_Y: src = norm_y; break;
    case PCD_GRID_PIXELS: src = pixels; break;
    case PCD_GRID_GRADIENT_X:
    case PCD_GRID_GRADIENT_Y: {
        // calculate_gradient(phi) (caustic_design.cpp:225), on request
        const size_t ng = (size_t)p.res_x * p.res_y;
        if (!grad) PCD_CUDA(cudaMalloc(&grad, 2 * ng * sizeof(double)));
        PCD_TRY(gradient(phi, grad, grad + ng, p.res_x, p.res_y, ctx->stream));
        src = which == PCD_GRID_GRADIENT_X ? grad : grad + ng;
        break;
    }
    default: set_error("pcd_design_get_grid: unknown grid"); return PCD_BAD_ARG;
    }
    cudaStream_t s = ctx->stream;
    PCD_CUDA(cudaMemcpyAsync(out, src, sizeof(double) * (size_t)p.res_x * p.res_y, cudaMemcpyDeviceToHost, s));
    PCD_CUDA(cudaStreamSynchronize(s));
    return PCD_OK;
}

int Design::get_vertices(int which, double *out)
{
    cudaStream_t s = ctx->stream;
    const int nx = p.mesh_res_x, ny = p.mesh_res_y, nv = nx * ny;
    const double *src = nullptr;
    switch (which) {
    case PCD_VERT_TARGET_POINTS:
    case PCD_VERT_SOURCE_POINTS:
    case PCD_VERT_CELL_POINTS:
        k_points_out<<<nblocks(nv), kT, 0, s>>>(which == PCD_VERT_CELL_POINTS ? tp_cells : tp, sz, nx, ny, p.width,
                                                 p.height, which == PCD_VERT_SOURCE_POINTS, pts_out);
        PCD_LAUNCHED(1);
        PCD_CUDA(cudaMemcpyAsync(out, pts_out, sizeof(double) * 3 * nv, cudaMemcpyDeviceToHost, s));
        PCD_CUDA(cudaStreamSynchronize(s));
        return PCD_OK;
    case PCD_VERT_INVERTED_MAP: {
        if (!initialized) {
            set_error("pcd_design_get_vertices: initialize first");
            return PCD_BAD_ARG;
        }
        PCD_TRY(locate(tp, 1, nx, ny, s));
        const QueryGrid g = query_grid(*this, 1);
        unsigned int *miss = (unsigned int *)small;
        PCD_CUDA(cudaMemsetAsync(miss, 0, sizeof(unsigned int), s));
        k_inverse_gather<<<nblocks(nv), kT, 0, s>>>(tp, g, owner, inv, miss);
        PCD_LAUNCHED(1);
        k_points_out<<<nblocks(nv), kT, 0, s>>>(inv, sz, nx, ny, p.width, p.height, false, pts_out);
        PCD_LAUNCHED(1);
        PCD_CUDA(cudaMemcpyAsync(small_host, miss, sizeof(unsigned int), cudaMemcpyDeviceToHost, s));
        PCD_CUDA(cudaMemcpyAsync(out, pts_out, sizeof(double) * 3 * nv, cudaMemcpyDeviceToHost, s));
        PCD_CUDA(cudaStreamSynchronize(s));
        if (*(unsigned int *)small_host) {
            set_error("inverse map miss: a source vertex lies in no deformed triangle");
            return PCD_RASTER_MISS;
        }
        return PCD_OK;
    }
    case PCD_VERT_TARGET_AREAS: src = target_areas; break;
    case PCD_VERT_ERRORS: src = errors; break;
    case PCD_VERT_NORMALS_X: src = nrm_x; break;
    case PCD_VERT_NORMALS_Y: src = nrm_y; break;
    case PCD_VERT_GRADIENT_X: src = vgx; break;
    case PCD_VERT_GRADIENT_Y: src = vgy; break;
    default: set_error("pcd_design_get_vertices: unknown field"); return PCD_BAD_ARG;
    }
    PCD_CUDA(cudaMemcpyAsync(out, src, sizeof(double) * nv, cudaMemcpyDeviceToHost, s));
    PCD_CUDA(cudaStreamSynchronize(s));
    return PCD_OK;
}

}  // namespace pcd
