/*
 * pcd_oracle.c -- CPU restatement of the reference's hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the checker that the CUDA library is
 * compared against; the product never links, loads or calls it.  Only tests/,
 * __graft_entry__.smoke() and bench.py's CPU-baseline leg use it.
 *
 * Every function restates one piece of dylanmsu/poisson_caustic_design and cites
 * the file:line it follows.  Arithmetic is plain IEEE double, written in the same
 * operation order as the reference, and the library is compiled with
 * -ffp-contract=off so that x86-64 and aarch64 builds give identical bits (the
 * reference itself is built without FMA contraction on x86-64).
 *
 * Parity pin: the SOR solver (pcdo_poisson_solver) is bit-identical to the
 * reference's poisson_solver() run with max_threads=1 (one tile, deterministic);
 * tests/test_oracle.py checks this against fixtures produced by the reference's
 * own compiled sources (oracle/_ref, see oracle/Makefile).
 *
 * Grids are row-major double arrays g[y*w + x] (the reference's
 * vector<vector<double>> g[y][x]); mesh points are n x 3 arrays (x, y, z).
 */
#include <math.h>
#include <pthread.h>
#include <stdlib.h>
#include <string.h>

/* ------------------------------------------------------------------------- */
/* Poisson solver: solver.cpp:12-61 (patial_relax) and :70-148               */
/* ------------------------------------------------------------------------- */

/* One lexicographic SOR sweep over the tile [x0,x1) x [y0,y1); returns the
 * largest |delta| (NaN deltas never raise it).  solver.cpp:12-61. */
static double relax_tile(double *phi, const double *b, int w, int h, double omega,
                         int x0, int y0, int x1, int y1)
{
    double max_update = 0.0;
    for (int y = y0; y < y1; y++) {
        for (int x = x0; x < x1; x++) {
            const long i = (long)y * w + x;
            double val = phi[i];
            double sum = 0.0, cnt = 0.0;
            /* neighbour order left, up, right, down (solver.cpp:29-44) */
            if (x != 0 && !isnan(b[i - 1])) { cnt += 1.0; sum += phi[i - 1]; }
            if (y != 0 && !isnan(b[i - w])) { cnt += 1.0; sum += phi[i - w]; }
            if (x != w - 1 && !isnan(b[i + 1])) { cnt += 1.0; sum += phi[i + 1]; }
            if (y != h - 1 && !isnan(b[i + w])) { cnt += 1.0; sum += phi[i + w]; }
            double delta = omega / cnt * (sum - cnt * val - b[i]);  /* solver.cpp:47 */
            double ad = fabs(delta);
            if (ad > max_update) max_update = ad;
            phi[i] += delta;
        }
    }
    return max_update;
}

/* poisson_solver(D, phi, width, height, max_iterations, tol, max_threads) with
 * max_threads in {1,2,3} (one tile).  solver.cpp:70-148.
 * Returns the number of sweeps run; *last_max_update gets the last sweep's max. */
int pcdo_poisson_solver(const double *b, double *phi, int w, int h, int max_iterations,
                        double tol, double *last_max_update)
{
    const double omega = 2.0 / (1.0 + 3.14159265 / w);   /* solver.cpp:71 */
    double mu = 0.0;
    int sweeps = 0;
    for (int i = 0; i < max_iterations; i++) {
        mu = relax_tile(phi, b, w, h, omega, 0, 0, w, h);
        sweeps = i + 1;
        if (mu < tol) break;                                /* solver.cpp:142 */
    }
    if (last_max_update) *last_max_update = mu;
    return sweeps;
}

/* The reference's threaded schedule, solver.cpp:70-148 with max_threads = T:
 * ceil/floor tiles on a floor(sqrt(min(T, hardware threads)))^2 grid
 * (:73-83, :121-131), one thread spawned per tile and joined every sweep, the
 * sweep's max |delta| taken under a mutex (:104-118).  Tiles read their
 * neighbours' boundary cells while those are being written, exactly like the
 * reference (chaotic relaxation), so results with T >= 4 are not bit-stable.
 * Returns the number of sweeps run. */
struct tile_job {
    double *phi;
    const double *b;
    int w, h, x0, y0, x1, y1;
    double omega;
    double *max_update;
    pthread_mutex_t *mtx;
};

static void *tile_worker(void *arg)
{
    struct tile_job *j = (struct tile_job *)arg;
    double m = relax_tile(j->phi, j->b, j->w, j->h, j->omega, j->x0, j->y0, j->x1, j->y1);
    pthread_mutex_lock(j->mtx);
    if (*j->max_update < m) *j->max_update = m;
    pthread_mutex_unlock(j->mtx);
    return NULL;
}

int pcdo_poisson_solver_threads(const double *b, double *phi, int w, int h, int max_iterations, double tol,
                                int max_threads, int hw_threads, double omega, double *last_max_update)
{
    if (omega <= 0.0) omega = 2.0 / (1.0 + 3.14159265 / w);   /* solver.cpp:71 */
    int nt = max_threads < hw_threads ? max_threads : hw_threads;
    int seg = (int)floor(sqrt((double)nt));
    if (seg < 1) seg = 1;
    int ntiles = seg * seg;
    struct tile_job *jobs = (struct tile_job *)malloc(sizeof(struct tile_job) * ntiles);
    pthread_t *th = (pthread_t *)malloc(sizeof(pthread_t) * ntiles);
    pthread_mutex_t mtx;
    pthread_mutex_init(&mtx, NULL);
    double mu = 0.0;
    int sweeps = 0;
    for (int i = 0; i < max_iterations; i++) {
        double max_update = 0.0;
        for (int ty = 0; ty < seg; ty++)
            for (int tx = 0; tx < seg; tx++) {
                struct tile_job *j = &jobs[ty * seg + tx];
                j->phi = phi; j->b = b; j->w = w; j->h = h; j->omega = omega;
                j->x0 = (int)floor((double)tx * ((double)w / (double)seg));
                j->y0 = (int)floor((double)ty * ((double)h / (double)seg));
                j->x1 = (int)ceil((double)(tx + 1) * ((double)w / (double)seg));
                j->y1 = (int)ceil((double)(ty + 1) * ((double)h / (double)seg));
                if (j->x1 > w) j->x1 = w;
                if (j->y1 > h) j->y1 = h;
                j->max_update = &max_update;
                j->mtx = &mtx;
            }
        if (ntiles == 1) {
            tile_worker(&jobs[0]);
        } else {
            for (int k = 0; k < ntiles; k++) pthread_create(&th[k], NULL, tile_worker, &jobs[k]);
            for (int k = 0; k < ntiles; k++) pthread_join(th[k], NULL);
        }
        mu = max_update;
        sweeps = i + 1;
        if (max_update < tol) break;
    }
    pthread_mutex_destroy(&mtx);
    free(jobs);
    free(th);
    if (last_max_update) *last_max_update = mu;
    return sweeps;
}

/* Same sweep with an explicit omega and no stop test: used by the CPU baseline
 * to run the reference's relaxation in fixed chunks.  Returns the last max. */
double pcdo_sor_sweeps(const double *b, double *phi, int w, int h, int sweeps, double omega)
{
    double mu = 0.0;
    for (int s = 0; s < sweeps; s++) mu = relax_tile(phi, b, w, h, omega, 0, 0, w, h);
    return mu;
}

/* r = b - L phi and its norms over cells whose b is not NaN; L is the Neumann
 * graph Laplacian of solver.cpp:29-47.  out[0]=||r||_2, out[1]=||b||_2,
 * out[2]=max|r|. */
void pcdo_residual(const double *b, const double *phi, int w, int h, double *r, double *out)
{
    double rr = 0.0, bb = 0.0, rmax = 0.0;
    for (int y = 0; y < h; y++) {
        for (int x = 0; x < w; x++) {
            const long i = (long)y * w + x;
            if (isnan(b[i])) { if (r) r[i] = NAN; continue; }
            double sum = 0.0, cnt = 0.0;
            if (x != 0 && !isnan(b[i - 1])) { cnt += 1.0; sum += phi[i - 1]; }
            if (y != 0 && !isnan(b[i - w])) { cnt += 1.0; sum += phi[i - w]; }
            if (x != w - 1 && !isnan(b[i + 1])) { cnt += 1.0; sum += phi[i + 1]; }
            if (y != h - 1 && !isnan(b[i + w])) { cnt += 1.0; sum += phi[i + w]; }
            double ri = b[i] - (sum - cnt * phi[i]);
            if (r) r[i] = ri;
            rr += ri * ri;
            bb += b[i] * b[i];
            if (fabs(ri) > rmax) rmax = fabs(ri);
        }
    }
    out[0] = sqrt(rr);
    out[1] = sqrt(bb);
    out[2] = rmax;
}

/* ------------------------------------------------------------------------- */
/* Grid utilities: utils.cpp                                                  */
/* ------------------------------------------------------------------------- */

/* subtractAverage: NaN-skipping mean removal, utils.cpp:60-86. */
void pcdo_subtract_average(double *g, long n)
{
    double sum = 0.0;
    int count = 0;
    for (long i = 0; i < n; i++)
        if (!isnan(g[i])) { sum += g[i]; count++; }
    double avg = sum / count;
    for (long i = 0; i < n; i++)
        if (!isnan(g[i])) g[i] = g[i] - avg;
}

/* calculate_gradient: central differences with clamped ends, utils.cpp:3-20. */
void pcdo_gradient(const double *g, int w, int h, double *gx, double *gy)
{
    for (int y = 0; y < h; y++) {
        for (int x = 0; x < w; x++) {
            int xp = x + 1 < w - 1 ? x + 1 : w - 1, xm = x - 1 > 0 ? x - 1 : 0;
            int yp = y + 1 < h - 1 ? y + 1 : h - 1, ym = y - 1 > 0 ? y - 1 : 0;
            gx[(long)y * w + x] = (g[(long)y * w + xp] - g[(long)y * w + xm]) / 2.0;
            gy[(long)y * w + x] = (g[(long)yp * w + x] - g[(long)ym * w + x]) / 2.0;
        }
    }
}

/* calculate_divergence: d(Nx)/dx + d(Ny)/dy, zero on the outer ring,
 * utils.cpp:22-39 (built on calculate_gradient). */
void pcdo_divergence(const double *nx, const double *ny, int w, int h, double *div)
{
    for (int y = 0; y < h; y++) {
        for (int x = 0; x < w; x++) {
            const long i = (long)y * w + x;
            if (x == 0 || x == w - 1 || y == 0 || y == h - 1) { div[i] = 0.0; continue; }
            double dx = (nx[i + 1] - nx[i - 1]) / 2.0;
            double dy = (ny[i + w] - ny[i - w]) / 2.0;
            div[i] = dx + dy;
        }
    }
}

/* scale_matrix_proportional: NaN-skipping min/max rescale to [lo, hi],
 * utils.cpp:88-129 (min/max seeded from element 0). */
void pcdo_scale_proportional(const double *in, long n, double lo, double hi, double *out)
{
    double mn = in[0], mx = in[0];
    for (long i = 0; i < n; i++)
        if (!isnan(in[i])) { mn = fmin(mn, in[i]); mx = fmax(mx, in[i]); }
    for (long i = 0; i < n; i++)
        out[i] = isnan(in[i]) ? 0.0 : lo + (hi - lo) * (in[i] - mn) / (mx - mn);
}

/* resize_image: nearest neighbour with integer source index, main.cpp:13-27. */
void pcdo_resize_nearest(const double *in, int ow, int oh, double *out, int nw, int nh)
{
    for (int y = 0; y < nh; y++)
        for (int x = 0; x < nw; x++)
            out[(long)y * nw + x] = in[(long)(y * oh / nh) * ow + (x * ow / nw)];
}

/* bilinearInterpolation with floor/ceil corners clamped to the image,
 * caustic_design.cpp:151-188. */
double pcdo_bilinear(const double *img, int w, int h, double x, double y)
{
    int x0 = (int)floor(x), y0 = (int)floor(y), x1 = (int)ceil(x), y1 = (int)ceil(y);
    x0 = x0 < 0 ? 0 : (x0 > w - 1 ? w - 1 : x0);
    x1 = x1 < 0 ? 0 : (x1 > w - 1 ? w - 1 : x1);
    y0 = y0 < 0 ? 0 : (y0 > h - 1 ? h - 1 : y0);
    y1 = y1 < 0 ? 0 : (y1 > h - 1 ? h - 1 : y1);
    double fx1 = x - x0, fx0 = 1.0 - fx1;
    double fy1 = y - y0, fy0 = 1.0 - fy1;
    double top = fx0 * img[(long)y0 * w + x0] + fx1 * img[(long)y0 * w + x1];
    double bot = fx0 * img[(long)y1 * w + x0] + fx1 * img[(long)y1 * w + x1];
    return fy0 * top + fy1 * bot;
}

/* ------------------------------------------------------------------------- */
/* Structured mesh: mesh.cpp                                                  */
/* ------------------------------------------------------------------------- */

/* generate_structured_mesh, mesh.cpp:45-64.  Triangle t of cell (i,j),
 * c = i*(nx-1)+j: t=2c is (v, v+1, v+nx), t=2c+1 is (v+nx, v+1, v+nx+1),
 * v = i*nx+j. */
void pcdo_mesh_points(int nx, int ny, double width, double height, double *pts)
{
    for (int i = 0; i < ny; i++)
        for (int j = 0; j < nx; j++) {
            double *p = pts + 3L * (i * nx + j);
            p[0] = (double)j * width / (nx - 1);
            p[1] = (double)i * height / (ny - 1);
            p[2] = 0.0;
        }
}

static inline void tri_vertices(int t, int nx, int v[3])
{
    int c = t >> 1, i = c / (nx - 1), j = c % (nx - 1), base = i * nx + j;
    if ((t & 1) == 0) { v[0] = base; v[1] = base + 1; v[2] = base + nx; }
    else { v[0] = base + nx; v[1] = base + 1; v[2] = base + nx + 1; }
}

/* Signed shoelace area of the quad (v, mid(v,j), centroid(v,j,k), mid(v,k)):
 * get_triangle_quad mesh.cpp:154-199 and calculate_polygon_area_vec
 * polygon_utils.cpp:194-214. */
static double quad_area(const double *pts, int vi, int vj, int vk)
{
    const double *a = pts + 3L * vi, *b = pts + 3L * vj, *c = pts + 3L * vk;
    double q[4][2];
    q[0][0] = a[0]; q[0][1] = a[1];
    q[1][0] = (a[0] + b[0]) / 2.0; q[1][1] = (a[1] + b[1]) / 2.0;
    q[2][0] = (a[0] + b[0] + c[0]) / 3.0; q[2][1] = (a[1] + b[1] + c[1]) / 3.0;
    q[3][0] = (a[0] + c[0]) / 2.0; q[3][1] = (a[1] + c[1]) / 2.0;
    double s = 0.0;
    for (int e = 0; e < 4; e++) {
        int f = (e + 1) & 3;
        s += q[e][0] * q[f][1] - q[f][0] * q[e][1];
    }
    return 0.5 * s;
}

/* Enumerate the (up to six) triangles around vertex (i,j) with the position of
 * the vertex inside each; same set as build_vertex_to_triangles mesh.cpp:106-118. */
static int vertex_triangles(int i, int j, int nx, int ny, int tri[6], int pos[6])
{
    int n = 0, cx = nx - 1;
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

/* Barycentric dual-cell areas: build_target_partitioned_dual_cells
 * mesh.cpp:201-231 + get_partitioned_source_areas polygon_utils.cpp:401-414.
 * (The reference sums the quads in hash-set order; the sum here runs in the
 * fixed order above, which changes only the last bits.) */
void pcdo_dual_cell_areas(const double *pts, int nx, int ny, double *areas)
{
    for (int i = 0; i < ny; i++)
        for (int j = 0; j < nx; j++) {
            int tri[6], pos[6], n = vertex_triangles(i, j, nx, ny, tri, pos);
            double a = 0.0;
            for (int k = 0; k < n; k++) {
                int v[3];
                tri_vertices(tri[k], nx, v);
                a += quad_area(pts, v[pos[k]], v[(pos[k] + 1) % 3], v[(pos[k] + 2) % 3]);
            }
            areas[i * nx + j] = a;
        }
}

/* Clip a convex polygon against the half plane s*(coord - c) >= 0 (axis 0=x,
 * 1=y).  Points on the line are kept; crossings are interpolated. */
static int clip_half(const double (*in)[2], int n, double (*out)[2], int axis, double c, double s)
{
    int m = 0;
    for (int k = 0; k < n; k++) {
        const double *p = in[k], *q = in[(k + 1) % n];
        double dp = s * (p[axis] - c), dq = s * (q[axis] - c);
        if (dp >= 0) { out[m][0] = p[0]; out[m][1] = p[1]; m++; }
        if ((dp > 0 && dq < 0) || (dp < 0 && dq > 0)) {
            double t = dp / (dp - dq);
            out[m][0] = p[0] + t * (q[0] - p[0]);
            out[m][1] = p[1] + t * (q[1] - p[1]);
            out[m][axis] = c;
            m++;
        }
    }
    return m;
}

static double poly_area(const double (*p)[2], int n)
{
    if (n < 3) return 0.0;
    double s = 0.0;
    for (int k = 0; k < n; k++) {
        int f = (k + 1) % n;
        s += p[k][0] * p[f][1] - p[f][0] * p[k][1];
    }
    return 0.5 * s;
}

/* Image-weighted area of one quad: integrate_cell_intensities
 * polygon_utils.cpp:311-366 (pixel side = width/image_w for both axes, pixel
 * range [floor(min/px), ceil(max/px)) clipped to the image).  The clipper is
 * our own Sutherland-Hodgman against the pixel's four half planes. */
static double quad_intensity(const double *img, int iw, int ih, double width, const double q[4][2])
{
    double xmin = q[0][0], xmax = q[0][0], ymin = q[0][1], ymax = q[0][1];
    for (int k = 1; k < 4; k++) {
        xmin = fmin(xmin, q[k][0]); xmax = fmax(xmax, q[k][0]);
        ymin = fmin(ymin, q[k][1]); ymax = fmax(ymax, q[k][1]);
    }
    double px = width / (double)iw, acc = 0.0;
    int ylo = (int)fmax(floor(ymin / px), 0.0), yhi = (int)fmin(ceil(ymax / px), (double)ih);
    int xlo = (int)fmax(floor(xmin / px), 0.0), xhi = (int)fmin(ceil(xmax / px), (double)iw);
    for (int y = ylo; y < yhi; y++)
        for (int x = xlo; x < xhi; x++) {
            double cx = ((double)x + 0.5) * px, cy = ((double)y + 0.5) * px;
            double a[12][2], b2[12][2];
            int n = clip_half(q, 4, a, 0, cx - px / 2.0, 1.0);
            n = clip_half((const double (*)[2])a, n, b2, 0, cx + px / 2.0, -1.0);
            n = clip_half((const double (*)[2])b2, n, a, 1, cy - px / 2.0, 1.0);
            n = clip_half((const double (*)[2])a, n, b2, 1, cy + px / 2.0, -1.0);
            acc += poly_area((const double (*)[2])b2, n) * img[(long)y * iw + x];
        }
    return acc;
}

/* get_target_partitioned_areas, polygon_utils.cpp:368-389: per-vertex image
 * integral over its dual cell, scaled so that the sum is width*height. */
void pcdo_target_areas(const double *img, int iw, int ih, double width, double height,
                       const double *pts, int nx, int ny, double *out)
{
    double total = 0.0;
    for (int i = 0; i < ny; i++)
        for (int j = 0; j < nx; j++) {
            int tri[6], pos[6], n = vertex_triangles(i, j, nx, ny, tri, pos);
            double a = 0.0;
            for (int k = 0; k < n; k++) {
                int v[3];
                tri_vertices(tri[k], nx, v);
                const double *A = pts + 3L * v[pos[k]], *B = pts + 3L * v[(pos[k] + 1) % 3],
                             *C = pts + 3L * v[(pos[k] + 2) % 3];
                double q[4][2] = {{A[0], A[1]},
                                  {(A[0] + B[0]) / 2.0, (A[1] + B[1]) / 2.0},
                                  {(A[0] + B[0] + C[0]) / 3.0, (A[1] + B[1] + C[1]) / 3.0},
                                  {(A[0] + C[0]) / 2.0, (A[1] + C[1]) / 2.0}};
                a += quad_intensity(img, iw, ih, width, q);
            }
            out[i * nx + j] = a;
            total += a;
        }
    double s = (width * height) / total;
    for (long k = 0; k < (long)nx * ny; k++) out[k] *= s;
}

/* Barycentric coordinates as bvh.cpp:162-190 computes them for the triangle
 * (t0,t1,t2) = (tri[2], tri[1], tri[0]); returns 1 when the point passes the
 * +-1e-12 acceptance test of bvh.cpp:208-217.  bc[k] weights tri vertex k. */
static int bary(const double *A, const double *B, const double *C, double px, double py, double bc[3])
{
    /* t0 = C, t1 = B, t2 = A */
    double v0x = A[0] - C[0], v0y = A[1] - C[1];
    double v1x = B[0] - C[0], v1y = B[1] - C[1];
    double v2x = px - C[0], v2y = py - C[1];
    double d00 = v0x * v0x + v0y * v0y, d01 = v0x * v1x + v0y * v1y, d02 = v0x * v2x + v0y * v2y;
    double d11 = v1x * v1x + v1y * v1y, d12 = v1x * v2x + v1y * v2y;
    double denom = d00 * d11 - d01 * d01;
    double inv = 1 / denom;
    double u = (d11 * d02 - d01 * d12) * inv;
    double v = (d00 * d12 - d01 * d02) * inv;
    double eps = 1e-12;
    bc[0] = u; bc[1] = v; bc[2] = 1.0 - u - v;
    return (u >= -eps && v >= -eps) && ((u + v) <= 1.0 + eps);
}

/* Sample grid of interpolate_raster_target/source, mesh.cpp:241-254. */
static inline double sample_coord(int i, int n, double extent)
{
    const double eps = 1e-8;
    return (double)i * (extent - eps) / (n - 1) + 0.5 * eps;
}

/* Mesh -> grid rasterisation by point location and barycentric interpolation:
 * interpolate_raster_target mesh.cpp:234-288 (and _source :291-345, which is the
 * same on the undeformed points).  Point location is our own scatter: every
 * triangle tests the samples inside its bounding box, and a sample takes the
 * lowest-numbered triangle that accepts it.  (The reference takes the first
 * hit of its BVH walk; hits differ only for samples on shared edges, where the
 * interpolants agree to rounding.)  Returns the number of samples no triangle
 * accepted; those are set to NaN (the reference calls exit(0) there). */
int pcdo_raster(const double *pts, const double *vals, int nx, int ny, double width,
                double height, int rx, int ry, double *out)
{
    long ns = (long)rx * ry;
    int *owner = (int *)malloc(sizeof(int) * ns);
    double *bcs = (double *)malloc(sizeof(double) * 3 * ns);
    for (long s = 0; s < ns; s++) owner[s] = -1;
    int ntri = 2 * (nx - 1) * (ny - 1);
    const double eps = 1e-8;
    for (int t = 0; t < ntri; t++) {
        int v[3];
        tri_vertices(t, nx, v);
        const double *A = pts + 3L * v[0], *B = pts + 3L * v[1], *C = pts + 3L * v[2];
        double xmin = fmin(A[0], fmin(B[0], C[0])), xmax = fmax(A[0], fmax(B[0], C[0]));
        double ymin = fmin(A[1], fmin(B[1], C[1])), ymax = fmax(A[1], fmax(B[1], C[1]));
        int ilo = (int)floor((xmin - 0.5 * eps) * (rx - 1) / (width - eps)) - 1;
        int ihi = (int)ceil((xmax - 0.5 * eps) * (rx - 1) / (width - eps)) + 1;
        int jlo = (int)floor((ymin - 0.5 * eps) * (ry - 1) / (height - eps)) - 1;
        int jhi = (int)ceil((ymax - 0.5 * eps) * (ry - 1) / (height - eps)) + 1;
        if (ilo < 0) ilo = 0;
        if (jlo < 0) jlo = 0;
        if (ihi > rx - 1) ihi = rx - 1;
        if (jhi > ry - 1) jhi = ry - 1;
        for (int jy = jlo; jy <= jhi; jy++) {
            double py = sample_coord(jy, ry, height);
            for (int ix = ilo; ix <= ihi; ix++) {
                long s = (long)jy * rx + ix;
                if (owner[s] >= 0) continue;      /* lower triangle already took it */
                double px = sample_coord(ix, rx, width), bc[3];
                if (bary(A, B, C, px, py, bc)) {
                    owner[s] = t;
                    bcs[3 * s] = bc[0]; bcs[3 * s + 1] = bc[1]; bcs[3 * s + 2] = bc[2];
                }
            }
        }
    }
    int misses = 0;
    for (long s = 0; s < ns; s++) {
        if (owner[s] < 0) { out[s] = NAN; misses++; continue; }
        int v[3];
        tri_vertices(owner[s], nx, v);
        out[s] = vals[v[0]] * bcs[3 * s] + vals[v[1]] * bcs[3 * s + 1] + vals[v[2]] * bcs[3 * s + 2];
    }
    free(owner);
    free(bcs);
    return misses;
}

/* calculate_inverted_transport_map, mesh.cpp:348-409: locate each (shrunk)
 * source vertex in the deformed target mesh, interpolate the source positions
 * there, and pin boundary vertices to their edges.  inv is n x 2.  Returns the
 * number of vertices not located (left as NaN). */
int pcdo_inverted_map(const double *tgt, const double *src, int nx, int ny, double width,
                      double height, double *inv)
{
    const double eps = 1e-8;
    long n = (long)nx * ny;
    int *owner = (int *)malloc(sizeof(int) * n);
    double *bcs = (double *)malloc(sizeof(double) * 3 * n);
    double *qx = (double *)malloc(sizeof(double) * n), *qy = (double *)malloc(sizeof(double) * n);
    for (long k = 0; k < n; k++) {
        owner[k] = -1;
        qx[k] = eps + src[3 * k] * ((width - 2 * eps) / width);
        qy[k] = eps + src[3 * k + 1] * ((height - 2 * eps) / height);
    }
    int ntri = 2 * (nx - 1) * (ny - 1);
    for (int t = 0; t < ntri; t++) {
        int v[3];
        tri_vertices(t, nx, v);
        const double *A = tgt + 3L * v[0], *B = tgt + 3L * v[1], *C = tgt + 3L * v[2];
        double xmin = fmin(A[0], fmin(B[0], C[0])), xmax = fmax(A[0], fmax(B[0], C[0]));
        double ymin = fmin(A[1], fmin(B[1], C[1])), ymax = fmax(A[1], fmax(B[1], C[1]));
        /* query k=(i,j) sits near (j*width/(nx-1), i*height/(ny-1)) */
        int jlo = (int)floor(xmin * (nx - 1) / width) - 1, jhi = (int)ceil(xmax * (nx - 1) / width) + 1;
        int ilo = (int)floor(ymin * (ny - 1) / height) - 1, ihi = (int)ceil(ymax * (ny - 1) / height) + 1;
        if (jlo < 0) jlo = 0;
        if (ilo < 0) ilo = 0;
        if (jhi > nx - 1) jhi = nx - 1;
        if (ihi > ny - 1) ihi = ny - 1;
        for (int i = ilo; i <= ihi; i++)
            for (int j = jlo; j <= jhi; j++) {
                long k = (long)i * nx + j;
                if (owner[k] >= 0) continue;
                double bc[3];
                if (bary(A, B, C, qx[k], qy[k], bc)) {
                    owner[k] = t;
                    bcs[3 * k] = bc[0]; bcs[3 * k + 1] = bc[1]; bcs[3 * k + 2] = bc[2];
                }
            }
    }
    int misses = 0;
    for (long k = 0; k < n; k++) {
        int i = (int)(k / nx), j = (int)(k % nx);
        if (owner[k] < 0) { inv[2 * k] = NAN; inv[2 * k + 1] = NAN; misses++; continue; }
        int v[3];
        tri_vertices(owner[k], nx, v);
        double ix = src[3L * v[0]] * bcs[3 * k] + src[3L * v[1]] * bcs[3 * k + 1] + src[3L * v[2]] * bcs[3 * k + 2];
        double iy = src[3L * v[0] + 1] * bcs[3 * k] + src[3L * v[1] + 1] * bcs[3 * k + 1] + src[3L * v[2] + 1] * bcs[3 * k + 2];
        int xe = (j == 0) ? -1 : (j == nx - 1 ? 1 : 0);
        int ye = (i == 0) ? -1 : (i == ny - 1 ? 1 : 0);
        inv[2 * k] = xe < 0 ? 0.0 : (xe > 0 ? width : ix);
        inv[2 * k + 1] = ye < 0 ? 0.0 : (ye > 0 ? height : iy);
    }
    free(owner); free(bcs); free(qx); free(qy);
    return misses;
}

/* calculate_refractive_normals_uniform, mesh.cpp:677-722: transmitted ray
 * t = normalize(inv - src_xy, focal - src_z), n = t - ri*(0,0,1), output the
 * slopes (nx/nz, ny/nz). */
void pcdo_refractive_normals(const double *inv, const double *src, long n, double focal,
                             double ri, double *nxo, double *nyo)
{
    for (long k = 0; k < n; k++) {
        double t0 = inv[2 * k] - src[3 * k], t1 = inv[2 * k + 1] - src[3 * k + 1];
        double t2 = 0 - src[3 * k + 2] + focal;
        double len = sqrt(t0 * t0 + t1 * t1 + t2 * t2);   /* normalize utils.cpp:370-384 */
        t0 /= len; t1 /= len; t2 /= len;
        double zx = t0 - 0.0 * ri, zy = t1 - 0.0 * ri, zz = t2 - 1.0 * ri;
        nxo[k] = zx / zz;
        nyo[k] = zy / zz;
    }
}

/* Mesh::step_grid mesh.cpp:485-532 plus the movement measure of
 * caustic_design.cpp:246-265.  Edge vertices slide along their edge, corners
 * are fixed, dt = width/res_x.  Returns max |dp| / width. */
double pcdo_step_grid(double *tgt, const double *vgx, const double *vgy, int nx, int ny,
                      double width, double step)
{
    double dt = width / nx, best = 0.0;
    for (int i = 0; i < ny; i++)
        for (int j = 0; j < nx; j++) {
            long k = (long)i * nx + j;
            int xedge = (j == 0 || j == nx - 1), yedge = (i == 0 || i == ny - 1);
            /* left/right edges keep only vy, top/bottom edges only vx */
            double vx = xedge ? 0.0 : vgx[k], vy = yedge ? 0.0 : vgy[k];
            double ox = tgt[3 * k], oy = tgt[3 * k + 1];
            tgt[3 * k] += vx * dt * step;
            tgt[3 * k + 1] += vy * dt * step;
            double dx = ox - tgt[3 * k], dy = oy - tgt[3 * k + 1], dz = 0.0;
            double d = sqrt(dx * dx + dy * dy + dz * dz);
            if (best < d) best = d;
        }
    return best / width;
}

/* Vertex sampling of the gradient at ((x/width)*rx - 0.5, (y/height)*ry - 0.5),
 * caustic_design.cpp:228-240; points is n x 3. */
void pcdo_sample_vertices(const double *grid, int rx, int ry, const double *pts, long n,
                          double width, double height, double *out)
{
    for (long k = 0; k < n; k++)
        out[k] = pcdo_bilinear(grid, rx, ry, (pts[3 * k] / width) * rx - 0.5,
                               (pts[3 * k + 1] / height) * ry - 0.5);
}

/* Mesh::set_source_heights mesh.cpp:724-742: subtract min(0, min h), store z,
 * return the sum of squared changes. */
double pcdo_set_source_heights(double *src, double *hv, long n)
{
    double m = 0;
    for (long k = 0; k < n; k++) if (m > hv[k]) m = hv[k];
    double s = 0.0;
    for (long k = 0; k < n; k++) {
        hv[k] -= m;
        s += (hv[k] - src[3 * k + 2]) * (hv[k] - src[3 * k + 2]);
        src[3 * k + 2] = hv[k];
    }
    return s;
}

/* Mesh::laplacian_smoothing mesh.cpp:534-606 on an nx x ny point set (n x 3):
 * corners stay; a left/right edge vertex takes the mean y of its three
 * neighbours (right or left, down, up -- in that order of summation), a
 * top/bottom edge vertex the mean x of its three (left, right, down / left,
 * up, right); interior vertices the mean x and y of left, right, up, down;
 * then p = mean * f + p * (1 - f).  The reference divides by 3.0f / 4.0f
 * (exact in double) and passes f as a float literal (0.1f). */
void pcdo_laplacian_smoothing(double *pts, int nx, int ny, double f)
{
    long n = (long)nx * ny;
    double *cp = (double *)malloc(sizeof(double) * 2 * n);
    for (long i = 0; i < n; i++) {
        int y = (int)(i / nx), x = (int)(i % nx);
        double px = pts[3 * i], py = pts[3 * i + 1];
#define P(yy, xx, c) pts[3 * ((long)(yy) * nx + (xx)) + (c)]
        int corner = (x == 0 || x == nx - 1) && (y == 0 || y == ny - 1);
        if (corner) {
        } else if (x == 0) {
            py = 0.0; py += P(y, x + 1, 1); py += P(y + 1, x, 1); py += P(y - 1, x, 1); py /= 3.0;
        } else if (x == nx - 1) {
            py = 0.0; py += P(y, x - 1, 1); py += P(y - 1, x, 1); py += P(y + 1, x, 1); py /= 3.0;
        } else if (y == 0) {
            px = 0.0; px += P(y, x - 1, 0); px += P(y, x + 1, 0); px += P(y + 1, x, 0); px /= 3.0;
        } else if (y == ny - 1) {
            px = 0.0; px += P(y, x - 1, 0); px += P(y - 1, x, 0); px += P(y, x + 1, 0); px /= 3.0;
        } else {
            px = 0.0; py = 0.0;
            px += P(y, x - 1, 0); px += P(y, x + 1, 0); px += P(y - 1, x, 0); px += P(y + 1, x, 0);
            py += P(y, x - 1, 1); py += P(y, x + 1, 1); py += P(y - 1, x, 1); py += P(y + 1, x, 1);
            px /= 4.0; py /= 4.0;
        }
#undef P
        cp[2 * i] = px;
        cp[2 * i + 1] = py;
    }
    for (long i = 0; i < n; i++) {
        pts[3 * i] = cp[2 * i] * f + pts[3 * i] * (1.0 - f);
        pts[3 * i + 1] = cp[2 * i + 1] * f + pts[3 * i + 1] * (1.0 - f);
    }
    free(cp);
}

/* Triangles of the structured mesh (mesh.cpp:57-63) whose signed area is
 * not positive: folds of the deformed target mesh. */
long pcdo_count_folds(const double *pts, int nx, int ny)
{
    long folds = 0;
    for (int y = 0; y < ny - 1; y++)
        for (int x = 0; x < nx - 1; x++) {
            long i = (long)y * nx + x;
            long t[2][3] = {{i, i + 1, i + nx}, {i + nx, i + 1, i + nx + 1}};
            for (int k = 0; k < 2; k++) {
                const double *a = pts + 3 * t[k][0], *b = pts + 3 * t[k][1], *c = pts + 3 * t[k][2];
                double area2 = (b[0] - a[0]) * (c[1] - a[1]) - (c[0] - a[0]) * (b[1] - a[1]);
                if (!(area2 > 0.0)) folds++;
            }
        }
    return folds;
}
