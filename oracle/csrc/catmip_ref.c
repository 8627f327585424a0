/*
 * FP64 C restatement of the CDM and Mogi data log-likelihood (oracle; CPU baseline).
 *
 * Test infrastructure only: used as the checker's fast path and to time the
 * CPU baseline.  Follows the reference numpy CDM models/cdm/cdm/libcdm.py:39-430
 * (the reference C++ models/cdm/lib/libcdm/cdm.cc needs GSL and disagrees with
 * the Matlab goldens) and the Mogi loop of models/mogi/lib/libmogi/Source.cc:65-118,
 * with the diagonal-Cd Gaussian log-likelihood norm - 1/2 Σ (r/σ)²
 * (models/cdm/cdm/Native.py:195-232).  Chains are split over POSIX threads.
 */
#include <math.h>
#include <pthread.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

typedef struct {
    int nparams, x_idx, depth_idx, strength_idx, axes_idx, omega_idx, log_strength;
    double nu;
} ref_layout;

typedef struct { double x, y, z; } v3;

static v3 vsub(v3 a, v3 b) { v3 r = {a.x - b.x, a.y - b.y, a.z - b.z}; return r; }
static v3 vadd(v3 a, v3 b) { v3 r = {a.x + b.x, a.y + b.y, a.z + b.z}; return r; }
static v3 vsc(v3 a, double s) { v3 r = {a.x * s, a.y * s, a.z * s}; return r; }
static double vdot(v3 a, v3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
static v3 vcross(v3 a, v3 b) {
    v3 r = {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
    return r;
}

/* libcdm.py:375-430 */
static void ang_dis(double y1, double y2, double beta, double b1, double b2, double b3, double nu,
                    double a, double* v1, double* v2, double* v3o) {
    const double sb = sin(beta), cb = cos(beta), cot = 1.0 / tan(beta), k = 1.0 - 2.0 * nu;
    const double z1 = y1 * cb + a * sb, z3 = y1 * sb - a * cb;
    const double r = sqrt(y1 * y1 + y2 * y2 + a * a);
    const double rpa = r + a, rmz = r - z3;
    const double fi = 2.0 * atan2(y2, rpa / tan(0.5 * beta) - y1);
    const double lpa = log(rpa), lmz = log(rmz);
    const double s = 0.5 / M_PI;
    double a1 = b1 * s * ((1 - k * cot * cot) * fi + y2 / rpa * (k * (cot + y1 / (2 * rpa)) - y1 / r) -
                          y2 * (r * sb - y1) * cb / (r * rmz));
    double a2 = b1 * s * (k * ((0.5 + cot * cot) * lpa - cot / sb * lmz) -
                          (k * (y1 * cot - 0.5 * a - y2 * y2 / (2 * rpa)) + y2 * y2 / r) / rpa +
                          y2 * y2 * cb / (r * rmz));
    double a3 = b1 * s * (k * fi * cot + y2 / rpa * (2 * nu + a / r) - y2 * cb / rmz * (cb + a / r));
    a1 += b2 * s * (-k * ((0.5 - cot * cot) * lpa + cot * cot * cb * lmz) -
                    (k * (y1 * cot + 0.5 * a + y1 * y1 / (2 * rpa)) - y1 * y1 / r) / rpa +
                    z1 * (r * sb - y1) / (r * rmz));
    a2 += b2 * s * ((1 + k * cot * cot) * fi - y2 / rpa * (k * (cot + y1 / (2 * rpa)) - y1 / r) -
                    y2 * z1 / (r * rmz));
    a3 += b2 * s * (-k * cot * (lpa - cb * lmz) - y1 / rpa * (2 * nu + a / r) + z1 / rmz * (cb + a / r));
    a1 += b3 * s * (y2 * (r * sb - y1) * sb / (r * rmz));
    a2 += b3 * s * (-y2 * y2 * sb / (r * rmz));
    a3 += b3 * s * (fi + y2 * (r * cb + a) * sb / (r * rmz));
    *v1 = a1; *v2 = a2; *v3o = a3;
}

/* one side PA->PB at one station, accumulated into (ue, un, uv) (libcdm.py:310-372) */
static void side_pair(double X, double Y, v3 b, v3 pa, v3 pb, double nu, double* ue, double* un,
                      double* uv) {
    v3 side = vsub(pb, pa);
    double L = sqrt(vdot(side, side));
    double beta = acos(-side.z / L);
    if (fabs(beta) < 2.220446049250313e-16 || fabs(M_PI - beta) < 2.220446049250313e-16) return;
    double hl = sqrt(side.x * side.x + side.y * side.y);
    double c = side.x / hl, s = side.y / hl;
    double y1a = c * (X - pa.x) + s * (Y - pa.y);
    double y2a = s * (X - pa.x) - c * (Y - pa.y);
    double y1b = y1a - (c * side.x + s * side.y);
    double y2b = y2a - (s * side.x - c * side.y);
    double b1 = c * b.x + s * b.y, b2 = s * b.x - c * b.y, b3 = -b.z;
    double be = (beta * y1a >= 0) ? beta - M_PI : beta;
    double va1, va2, va3, vb1, vb2, vb3;
    ang_dis(y1a, y2a, be, b1, b2, b3, nu, -pa.z, &va1, &va2, &va3);
    ang_dis(y1b, y2b, be, b1, b2, b3, nu, -pb.z, &vb1, &vb2, &vb3);
    double v1 = vb1 - va1, v2 = vb2 - va2, v3_ = vb3 - va3;
    *ue += c * v1 + s * v2;
    *un += s * v1 - c * v2;
    *uv += -v3_;
}

/* corners (libcdm.py:174-217); returns 1 if above the free surface */
static int corners(const double* th, const ref_layout* L, v3 V[3][4]) {
    double x0 = th[L->x_idx], y0 = th[L->x_idx + 1], depth = th[L->depth_idx];
    double lx = 2 * th[L->axes_idx], ly = 2 * th[L->axes_idx + 1], lz = 2 * th[L->axes_idx + 2];
    double d2r = M_PI / 180.0;
    double cx = cos(th[L->omega_idx] * d2r), sx = sin(th[L->omega_idx] * d2r);
    double cy = cos(th[L->omega_idx + 1] * d2r), sy = sin(th[L->omega_idx + 1] * d2r);
    double cz = cos(th[L->omega_idx + 2] * d2r), sz = sin(th[L->omega_idx + 2] * d2r);
    double ryx[3][3] = {{cy, sy * sx, -sy * cx}, {0, cx, sx}, {sy, -cy * sx, cy * cx}};
    double rz[3][3] = {{cz, sz, 0}, {-sz, cz, 0}, {0, 0, 1}};
    double R[3][3];
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) R[i][j] = rz[i][0] * ryx[0][j] + rz[i][1] * ryx[1][j] + rz[i][2] * ryx[2][j];
    v3 ex = {R[0][0], R[1][0], R[2][0]}, ey = {R[0][1], R[1][1], R[2][1]}, ez = {R[0][2], R[1][2], R[2][2]};
    v3 c0 = {x0, y0, -depth};
    V[0][0] = vadd(c0, vadd(vsc(ey, 0.5 * ly), vsc(ez, 0.5 * lz)));
    V[0][1] = vsub(V[0][0], vsc(ey, ly));
    V[0][2] = vsub(V[0][1], vsc(ez, lz));
    V[0][3] = vsub(V[0][0], vsc(ez, lz));
    V[1][0] = vadd(vsub(c0, vsc(ex, 0.5 * lx)), vsc(ez, 0.5 * lz));
    V[1][1] = vadd(V[1][0], vsc(ex, lx));
    V[1][2] = vsub(V[1][1], vsc(ez, lz));
    V[1][3] = vsub(V[1][0], vsc(ez, lz));
    V[2][0] = vadd(c0, vadd(vsc(ex, 0.5 * lx), vsc(ey, 0.5 * ly)));
    V[2][1] = vsub(V[2][0], vsc(ex, lx));
    V[2][2] = vsub(V[2][1], vsc(ey, ly));
    V[2][3] = vsub(V[2][0], vsc(ey, ly));
    for (int a = 0; a < 3; ++a)
        for (int b = 0; b < 4; ++b)
            if (V[a][b].z > 0) return 1;
    return 0;
}

/* LOS displacement of one CDM sample at m stations; returns 1 if above the surface */
int ref_cdm_los(const double* th, const ref_layout* L, const double* x, const double* y,
                const double* los, int m, double* out) {
    v3 V[3][4];
    if (corners(th, L, V)) return 1;
    double ax = th[L->axes_idx], ay = th[L->axes_idx + 1], az = th[L->axes_idx + 2];
    int use[3] = {1, 1, 1};
    if (ax == 0 && ay == 0 && az == 0) { use[0] = use[1] = use[2] = 0; }
    else if (ax == 0 && ay != 0 && az != 0) { use[1] = use[2] = 0; }
    else if (ax != 0 && ay == 0 && az != 0) { use[0] = use[2] = 0; }
    else if (ax != 0 && ay != 0 && az == 0) { use[0] = use[1] = 0; }
    v3 b[3];
    for (int r = 0; r < 3; ++r) {
        v3 n = vcross(vsub(V[r][1], V[r][0]), vsub(V[r][3], V[r][0]));
        b[r] = vsc(n, th[L->strength_idx] / sqrt(vdot(n, n)));
    }
    for (int j = 0; j < m; ++j) {
        double ue = 0, un = 0, uv = 0;
        for (int r = 0; r < 3; ++r) {
            if (!use[r]) continue;
            for (int e = 0; e < 4; ++e) side_pair(x[j], y[j], b[r], V[r][e], V[r][(e + 1) & 3], L->nu, &ue, &un, &uv);
        }
        out[j] = ue * los[3 * j] + un * los[3 * j + 1] + uv * los[3 * j + 2];
    }
    return 0;
}

/* Mogi LOS displacement (libmogi/Source.cc:73-113) */
void ref_mogi_los(const double* th, const ref_layout* L, const double* x, const double* y,
                  const double* los, int m, double* out) {
    double xs = th[L->x_idx], ys = th[L->x_idx + 1], d = th[L->depth_idx];
    double dv = L->log_strength ? pow(10.0, th[L->strength_idx]) : th[L->strength_idx];
    double C = (L->nu - 1) * dv / M_PI;
    for (int j = 0; j < m; ++j) {
        double dx = xs - x[j], dy = ys - y[j];
        double R = sqrt(dx * dx + dy * dy + d * d);
        out[j] = (dx * los[3 * j] + dy * los[3 * j + 1] - d * los[3 * j + 2]) * C / (R * R * R);
    }
}

typedef struct {
    int model; const double* theta; int lo, hi; const ref_layout* L;
    const double *x, *y, *los, *d, *w; int m; double norm; double* llk; int* invalid;
} job_t;

static void* worker(void* arg) {
    job_t* J = (job_t*)arg;
    double* u = (double*)malloc(sizeof(double) * (size_t)J->m);
    for (int i = J->lo; i < J->hi; ++i) {
        const double* th = J->theta + (size_t)i * J->L->nparams;
        int bad = 0;
        if (J->model == 2) bad = ref_cdm_los(th, J->L, J->x, J->y, J->los, J->m, u);
        else ref_mogi_los(th, J->L, J->x, J->y, J->los, J->m, u);
        if (J->invalid) J->invalid[i] = bad;
        if (bad) { J->llk[i] = -INFINITY; continue; }
        double s = 0;
        for (int j = 0; j < J->m; ++j) { double r = u[j] - J->d[j]; s += r * r * J->w[j]; }
        J->llk[i] = J->norm - 0.5 * s;
    }
    free(u);
    return NULL;
}

/* data log-likelihood of n samples; model 1 = Mogi, 2 = CDM; returns 0 */
int ref_llk(int model, const double* theta, int n, const ref_layout* L, const double* x,
            const double* y, const double* los, const double* d, const double* w, int m,
            double norm, double* llk, int* invalid, int nthreads) {
    if (nthreads < 1) nthreads = 1;
    if (nthreads > n) nthreads = n;
    pthread_t* tid = (pthread_t*)malloc(sizeof(pthread_t) * (size_t)nthreads);
    job_t* jobs = (job_t*)malloc(sizeof(job_t) * (size_t)nthreads);
    for (int t = 0; t < nthreads; ++t) {
        job_t J = {model, theta, (int)((long)n * t / nthreads), (int)((long)n * (t + 1) / nthreads), L,
                   x, y, los, d, w, m, norm, llk, invalid};
        jobs[t] = J;
        pthread_create(&tid[t], NULL, worker, &jobs[t]);
    }
    for (int t = 0; t < nthreads; ++t) pthread_join(tid[t], NULL);
    free(tid);
    free(jobs);
    return 0;
}
