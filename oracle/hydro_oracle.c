/*
 * hydro_oracle.c -- CPU parity oracle for the HydroGPU Euler Roe/HLLC/HLL step.
 *
 * TEST INFRASTRUCTURE ONLY: loaded by tests/, __graft_entry__.smoke() and the
 * CPU-baseline leg of bench.py as the checker; never linked into the product.
 *
 * Builds liboracle.so (gcc -O2 -ffp-contract=off -fopenmp).  The numerics live in
 * oracle_impl.h, instantiated here for double and float.  The host-side rules
 * restated here are the reference's program preamble (src/Solver/Solver.cpp:260-315):
 * DX/DY/DZ printed with std::stringstream's default 6 significant digits
 * (include/HydroGPU/toNumericString.h:12-22), the `defs` numbers printed the way
 * Lua prints numbers (%.14g), and dim = last axis with size > 1
 * (src/HydroGPUApp.cpp:214-221), dx = (xmax-xmin)/(float)size (:224-226).
 */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <tgmath.h>
#include <float.h>
#include <math.h>
#ifdef _OPENMP
#include <omp.h>
#endif
#include "../include/hgpu/hgpu.h"

/* dot(a,b) of two 4-vectors, summed x, y, z, w in that order */
#define DOT4(a, b) (((a)[0] * (b)[0] + (a)[1] * (b)[1]) + (a)[2] * (b)[2] + (a)[3] * (b)[3])

#define REAL double
#define REAL_MAX DBL_MAX
#define SFX_TOKEN f64
#include "oracle_impl.h"
#undef REAL
#undef REAL_MAX
#undef SFX_TOKEN

#define REAL float
#define REAL_MAX FLT_MAX
#define SFX_TOKEN f32
#include "oracle_impl.h"
#undef REAL
#undef REAL_MAX
#undef SFX_TOKEN

typedef struct oracle_handle {
    int precision;
    osolver_f64* d;
    osolver_f32* f;
} oracle_handle;

/* toNumericString<double>: ostream default (precision 6, %g-like) */
static double baked6(double v) {
    char buf[64];
    snprintf(buf, sizeof buf, "%g", v);
    return strtod(buf, NULL);
}

int oracle_resolve(const hgpu_config* cfg, int* dim_out, double dx[3], double* gamma_out, double* g_out) {
    if (!cfg) return HGPU_ERR_ARG;
    int dim = cfg->dim;
    if (dim == 0) {
        for (dim = 3; dim > 0; --dim)
            if (cfg->size[dim - 1] > 1) break;
    }
    if (dim < 1 || dim > 3) return HGPU_ERR_CONFIG;
    for (int i = 0; i < 3; ++i) {
        if (i < dim && cfg->size[i] < 5) return HGPU_ERR_CONFIG;
        if (i >= dim && cfg->size[i] != 1) return HGPU_ERR_CONFIG;
    }
    if (cfg->solver != HGPU_SOLVER_ROE && cfg->solver != HGPU_SOLVER_HLLC && cfg->solver != HGPU_SOLVER_HLL)
        return HGPU_ERR_CONFIG;
    if (cfg->limiter < 0 || cfg->limiter >= HGPU_NUM_LIMITERS) return HGPU_ERR_CONFIG;
    if (cfg->integrator < 0 || cfg->integrator >= HGPU_NUM_INTEGRATORS) return HGPU_ERR_CONFIG;
    for (int i = 0; i < 3; ++i) {
        double d;
        if (cfg->precision == HGPU_FP32) {
            float df = ((float)cfg->xmax[i] - (float)cfg->xmin[i]) / (float)cfg->size[i];
            d = (double)df;
        } else {
            d = (cfg->xmax[i] - cfg->xmin[i]) / (double)(float)cfg->size[i];
        }
        dx[i] = cfg->compat == HGPU_COMPAT_REF ? baked6(d) : d;
        if (i < dim && !(dx[i] > 0)) return HGPU_ERR_CONFIG;
    }
    if (cfg->gauss_seidel_max_iter < 0) return HGPU_ERR_CONFIG;
    {
        char buf[64];
        snprintf(buf, sizeof buf, "%.14g", cfg->gamma);
        *gamma_out = cfg->compat == HGPU_COMPAT_REF ? strtod(buf, NULL) : cfg->gamma;
        snprintf(buf, sizeof buf, "%.14g", cfg->gravitational_constant);
        *g_out = cfg->compat == HGPU_COMPAT_REF ? strtod(buf, NULL) : cfg->gravitational_constant;
    }
    *dim_out = dim;
    return HGPU_OK;
}

int oracle_create(const hgpu_config* cfg, oracle_handle** out) {
    int dim;
    double dx[3], gamma, G;
    int st = oracle_resolve(cfg, &dim, dx, &gamma, &G);
    if (st) return st;
    if (cfg->compat != HGPU_COMPAT_REF) return HGPU_ERR_UNSUPPORTED;
    oracle_handle* h = (oracle_handle*)calloc(1, sizeof *h);
    h->precision = cfg->precision;
    if (cfg->precision == HGPU_FP32) h->f = create_f32(cfg, dim, dx, gamma, G);
    else h->d = create_f64(cfg, dim, dx, gamma, G);
    *out = h;
    return HGPU_OK;
}

void oracle_destroy(oracle_handle* h) {
    if (!h) return;
    destroy_f64(h->d);
    destroy_f32(h->f);
    free(h);
}

size_t oracle_count(const oracle_handle* h) {
    return h->d ? (size_t)h->d->V * h->d->N : (size_t)h->f->V * h->f->N;
}

/* Solver::resetState's upload: the state, then SelfGravitation::resetState with the
 * initial conditions' potential channel (pot: one value per cell, or NULL = zero). */
int oracle_set_state_potential(oracle_handle* h, const void* src, size_t count, const void* pot, size_t pcount) {
    if (!h || !src || count != oracle_count(h)) return HGPU_ERR_ARG;
    if (pot && pcount != (size_t)(h->d ? h->d->V : h->f->V)) return HGPU_ERR_ARG;
    if (h->d) {
        memcpy(h->d->state, src, count * sizeof(double));
        resetPotential_f64(h->d, (const double*)pot);
    } else {
        memcpy(h->f->state, src, count * sizeof(float));
        resetPotential_f32(h->f, (const float*)pot);
    }
    return HGPU_OK;
}

int oracle_set_state(oracle_handle* h, const void* src, size_t count) {
    return oracle_set_state_potential(h, src, count, NULL, 0);
}

int oracle_get_potential(oracle_handle* h, void* dst, size_t count) {
    if (!h || !dst || count != (size_t)(h->d ? h->d->V : h->f->V)) return HGPU_ERR_ARG;
    if (h->d) memcpy(dst, h->d->potential, count * sizeof(double));
    else memcpy(dst, h->f->potential, count * sizeof(float));
    return HGPU_OK;
}

int oracle_get_state(oracle_handle* h, void* dst, size_t count) {
    if (!h || !dst || count != oracle_count(h)) return HGPU_ERR_ARG;
    if (h->d) memcpy(dst, h->d->state, count * sizeof(double));
    else memcpy(dst, h->f->state, count * sizeof(float));
    return HGPU_OK;
}

/* nsteps x Solver::update; *last_dt = dt of the last step; *nonfinite = a NaN was
 * seen in the CFL reduction in any step. */
int oracle_update(oracle_handle* h, int nsteps, double* last_dt, int* nonfinite) {
    if (!h || nsteps < 0) return HGPU_ERR_ARG;
    int bad = 0;
    for (int n = 0; n < nsteps; ++n) {
        int b = 0;
        if (h->d) update_f64(h->d, &b);
        else update_f32(h->f, &b);
        bad |= b;
    }
    if (last_dt) *last_dt = h->d ? h->d->lastDt : h->f->lastDt;
    if (nonfinite) *nonfinite = bad;
    return HGPU_OK;
}

/* The display scalar of every cell (convertToTex); method = the reference's DISPLAY_* index. */
int oracle_display(oracle_handle* h, int method, float* out) {
    if (!h || !out) return HGPU_ERR_ARG;
    return h->d ? display_f64(h->d, method, out) : display_f32(h->f, method, out);
}

/* Copy an internal buffer out (per-kernel checks): "eigenvalues", "flux", "dt". */
size_t oracle_get_buffer(oracle_handle* h, const char* name, void* out, size_t cap) {
    size_t n = 0;
    const void* src = NULL;
    size_t es = h->d ? sizeof(double) : sizeof(float);
    long V = h->d ? h->d->V : h->f->V;
    int N = h->d ? h->d->N : h->f->N, D = h->d ? h->d->dim : h->f->dim;
    if (!strcmp(name, "eigenvalues")) { n = (size_t)V * D * N; src = h->d ? (void*)h->d->eigenvalues : (void*)h->f->eigenvalues; }
    else if (!strcmp(name, "flux")) { n = (size_t)V * D * N; src = h->d ? (void*)h->d->flux : (void*)h->f->flux; }
    else if (!strcmp(name, "dt")) { n = (size_t)V * D; src = h->d ? (void*)h->d->dtBuffer : (void*)h->f->dtBuffer; }
    if (!src) return 0;
    if (out && cap >= n) memcpy(out, src, n * es);
    return n;
}

void oracle_set_threads(int n) {
#ifdef _OPENMP
    if (n > 0) omp_set_num_threads(n);
#else
    (void)n;
#endif
}

int oracle_max_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}
