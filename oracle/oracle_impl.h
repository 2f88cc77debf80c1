/*
 * oracle_impl.h -- CPU restatement of HydroGPU's Euler Roe/HLLC update.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the parity oracle: it is compiled into
 * oracle/liboracle.so and may be loaded only by tests/, __graft_entry__.smoke()
 * and the CPU-baseline leg of bench.py.  The product (libhgpu.so) never links it.
 *
 * It restates, buffer for buffer, what the reference's OpenCL kernels do when
 * driven in the reference host order, with every never-written buffer entry
 * defined as zero (fresh allocation).  It is included twice by hydro_oracle.c,
 * with REAL = double and REAL = float.  Compile with -ffp-contract=off so that
 * every a*b+c is two roundings, like the reference kernels' source.
 *
 * Reference citations are path:line inside KennethYeah/HydrodynamicsGPU.
 */

#ifndef ORACLE_IMPL_COMMON
#define ORACLE_IMPL_COMMON
#define FN_CAT2(a, b) a##_##b
#define FN_CAT(a, b) FN_CAT2(a, b)
#define FN(name) FN_CAT(name, SFX_TOKEN)
#define IDX(s, x, y, z) ((long)(x) + (long)(s)->S[0] * ((long)(y) + (long)(s)->S[1] * (long)(z)))
#define FOR_CELLS(s)                                    \
    _Pragma("omp parallel for collapse(2) schedule(static)") \
    for (int z = 0; z < (s)->S[2]; ++z)                 \
        for (int y = 0; y < (s)->S[1]; ++y)             \
            for (int x = 0; x < (s)->S[0]; ++x)
enum { BK_PERIODIC = 0, BK_MIRROR, BK_REFLECT, BK_FREEFLOW };
enum { CB_FLUX = 0, CB_GRAVITY = 1 };
#endif

typedef struct {
    hgpu_config cfg;
    int dim, N, S[3], step[3];
    long V;
    REAL dx[3];        /* DX/DY/DZ as baked into the program (Solver.cpp:272-274) */
    REAL gamma;        /* ((real)<defs value>) (Solver.cpp:298)                  */
    REAL G;            /* selfGrav_gravitationalConstant = ((real)<defs value>)  */
    float cfl;
    int isHLLC;        /* an HLL-family solver (EulerHLLC or EulerHLL): HLL.cpp driver */
    int isHLL;         /* EulerHLL: Davis-bounded wave speeds, two-state HLL flux     */
    REAL* state;       /* Solver::stateBuffer                                     */
    REAL* potential;   /* SelfGravitation::potentialBuffer                        */
    REAL* eigenvalues; /* Roe: V*dim*N; HLL: V*dim*N                               */
    REAL* eigenvectors;/* Roe: V*dim*2*N*N (first N*N = left/inverse, then right) */
    REAL* deltaQTilde; /* Roe: V*dim*N                                            */
    REAL* flux;        /* FiniteVolumeSolver::fluxBuffer, zeroed (FiniteVolumeSolver.cpp:14) */
    REAL* dtBuffer;    /* V*dim, initialised to REAL_MAX (Solver.cpp:217-222)     */
    /* integrator buffers (RungeKutta.h:97-125 / ForwardEuler.cpp:8-17) */
    REAL* sb[4];
    REAL* db[4];
    double lastDt;
    REAL lastDtReal;
} FN(osolver);

/* ---------------- tableaus: include/HydroGPU/Integrator/RungeKutta.h:129-294 ---------------- */
static int FN(tableau)(int integ, REAL alpha[4][4], REAL beta[4][4]) {
    static const double A[HGPU_NUM_INTEGRATORS][4][4] = {
        /* FE (unused) */ {{0}},
        /* RK2 :129-140 */ {{1, 0}, {1, 0}},
        /* RK2Heun :142-153 */ {{1, 0}, {1, 0}},
        /* RK2Ralston :155-166 */ {{1, 0}, {1, 0}},
        /* RK3 :168-181 */ {{1, 0, 0}, {1, 0, 0}, {1, 0, 0}},
        /* RK4 :183-198 */ {{1, 0, 0, 0}, {1, 0, 0, 0}, {1, 0, 0, 0}, {1, 0, 0, 0}},
        /* RK4 3/8 :200-215 */ {{1, 0, 0, 0}, {1, 0, 0, 0}, {1, 0, 0, 0}, {1, 0, 0, 0}},
        /* RK2TVD :219-230 */ {{1, 0}, {.5, .5}},
        /* RK2NonTVD :232-243 */ {{1, 0}, {1, 0}},
        /* RK3TVD :245-258 */ {{1, 0, 0}, {3. / 4., 1. / 4., 0}, {1. / 3., 2. / 3., 0}},
        /* RK4TVD :260-275 */ {{1, 0, 0, 0}, {649. / 1600., 951. / 1600., 0, 0},
                                {53989. / 2500000., 4806213. / 20000000., 23619. / 32000., 0},
                                {1. / 5., 6127. / 30000., 7873. / 30000., 1. / 3.}},
        /* RK4NonTVD :279-294 */ {{1, 0, 0, 0}, {1, 0, 0, 0}, {1, 0, 0, 0}, {-1. / 3., 1. / 3., 2. / 3., 1. / 3.}},
    };
    static const double B[HGPU_NUM_INTEGRATORS][4][4] = {
        {{0}},
        {{.5, 0}, {0, 1}},
        {{1, 0}, {.5, .5}},
        {{2. / 3., 0}, {1. / 4., 3. / 4.}},
        {{.5, 0, 0}, {-1, 2, 0}, {1. / 6., 2. / 6., 1. / 6.}},
        {{.5, 0, 0, 0}, {0, .5, 0, 0}, {0, 0, 1, 0}, {1. / 6., 2. / 6., 2. / 6., 1. / 6.}},
        {{1. / 3., 0, 0, 0}, {-1. / 3., 0, 0, 0}, {1, -1, 1, 0}, {1. / 8., 3. / 8., 3. / 8., 1. / 8.}},
        {{1, 0}, {0, .5}},
        {{-20, 0}, {41. / 40., -1. / 40.}},
        {{1, 0, 0}, {0, 1. / 4., 0}, {0, 0, 2. / 3.}},
        {{.5, 0, 0, 0}, {-10890423. / 25193600., 5000. / 7873, 0, 0},
         {-102261. / 5000000., -5121. / 20000., 7873. / 10000., 0}, {1. / 10., 1. / 6., 0, 1. / 6.}},
        {{.5, 0, 0, 0}, {0, .5, 0, 0}, {0, 0, 1, 0}, {0, 0, 0, 1. / 6.}},
    };
    static const int order[HGPU_NUM_INTEGRATORS] = {1, 2, 2, 2, 3, 4, 4, 2, 2, 3, 4, 4};
    for (int i = 0; i < 4; ++i)
        for (int j = 0; j < 4; ++j) {
            alpha[i][j] = (REAL)A[integ][i][j];
            beta[i][j] = (REAL)B[integ][i][j];
        }
    return order[integ];
}

/* ---------------- slope limiters: res/SlopeLimiter.cl:5-68 ----------------
 * OpenCL min/max are taken with fmin/fmax semantics (a NaN argument yields the
 * other argument); the arithmetic order is that of the source expressions. */
static REAL FN(slopeLimiter)(int lim, REAL r) {
    switch (lim) {
    case HGPU_LIMITER_DONORCELL: return 0.;                                      /* :6-8   */
    case HGPU_LIMITER_LAXWENDROFF: return 1.;                                    /* :9-11  */
    case HGPU_LIMITER_BEAMWARMING: return r;                                     /* :12-14 */
    case HGPU_LIMITER_FROMM: return (REAL)(.5 * (1. + r));                       /* :15-17 */
    case HGPU_LIMITER_CHARM:                                                     /* :18-20 */
        return (REAL)((REAL)fmax((REAL)0., (REAL)r) * (3. * r + 1.) / ((r + 1.) * (r + 1.)));
    case HGPU_LIMITER_HCUS:                                                      /* :21-23 */
        return (REAL)fmax((REAL)0., (REAL)(1.5 * (r + (REAL)fabs(r)) / (r + 2.)));
    case HGPU_LIMITER_HQUICK:                                                    /* :24-26 */
        return (REAL)fmax((REAL)0., (REAL)(2. * (r + (REAL)fabs(r)) / (r + 3.)));
    case HGPU_LIMITER_KOREN:                                                     /* :27-29 */
        return (REAL)fmax((REAL)0., (REAL)fmin(2. * r, (REAL)fmin((1. + 2. * r) / 3., 2.)));
    case HGPU_LIMITER_MINMOD:                                                    /* :30-32 */
        return (REAL)fmax((REAL)0., (REAL)fmin(r, (REAL)1.));
    case HGPU_LIMITER_OSHKER:                                                    /* :33-35 */
        return (REAL)fmax((REAL)0., (REAL)fmin(r, (REAL)1.5));
    case HGPU_LIMITER_OSPRE:                                                     /* :36-38 */
        return (REAL)(.5 * (r * r + r) / (r * r + r + 1.));
    case HGPU_LIMITER_SMART:                                                     /* :39-41 */
        return (REAL)fmax((REAL)0., (REAL)fmin(2. * r, (REAL)fmin(.25 + .75 * r, 4.)));
    case HGPU_LIMITER_SWEBY:                                                     /* :42-44 */
        return (REAL)fmax((REAL)0., (REAL)fmax((REAL)fmin(1.5 * r, 1.), (REAL)fmin(r, 1.5)));
    case HGPU_LIMITER_UMIST:                                                     /* :45-47 */
        return (REAL)fmax((REAL)0., (REAL)fmin((REAL)fmin(2. * r, .75 + .25 * r), (REAL)fmin(.25 + .75 * r, 2.)));
    case HGPU_LIMITER_VANALBADA1: return (REAL)((r * r + r) / (r * r + 1.));     /* :48-50 */
    case HGPU_LIMITER_VANALBADA2: return (REAL)(2. * r / (r * r + 1.));          /* :51-53 */
    case HGPU_LIMITER_VANLEER:                                                   /* :54-58 */
        return (REAL)((REAL)fmax((REAL)0., r) * 2. / (1. + r));
    case HGPU_LIMITER_MONOTIZEDCENTRAL:                                          /* :59-61 */
        return (REAL)fmax((REAL)0., (REAL)fmin(2., (REAL)fmin(.5 * (1. + r), 2. * r)));
    case HGPU_LIMITER_SUPERBEE:                                                  /* :62-64 */
        return (REAL)fmax((REAL)0., (REAL)fmax((REAL)fmin((REAL)1., (REAL)2. * r), (REAL)fmin((REAL)2., (REAL)r)));
    case HGPU_LIMITER_BARTHJESPERSEN:                                            /* :65-67 */
        return (REAL)(.5 * (r + 1.) * (REAL)fmin((REAL)1., (REAL)fmin(4. * r / (r + 1.), 4. / (r + 1.))));
    }
    return 0.;
}

/* true when every active coordinate lies in [lo, S-hi) */
static inline int FN(inRange)(const FN(osolver) * s, int x, int y, int z, int lo, int hi) {
    if (x < lo || x >= s->S[0] - hi) return 0;
    if (s->dim > 1 && (y < lo || y >= s->S[1] - hi)) return 0;
    if (s->dim > 2 && (z < lo || z >= s->S[2] - hi)) return 0;
    return 1;
}

/* ---------------- boundary: Solver::boundary (Solver.cpp:448-464), kernels Common.cl:49-194 ----------------
 * Axis-major, then state, then min before max.  Mirror uses Reflect on the
 * normal momentum (Euler.cpp:63-75).  In 1D the Mirror/Reflect/FreeFlow kernels
 * have no range guard and their work-items k>0 address INDEX(0,k,0), outside
 * the buffer; only the in-bounds work-item 0 is restated. */
static void FN(boundaryKernel)(FN(osolver) * s, REAL* buf, int spacing, int offset, int kernel, int axis, int minmax) {
    int S0 = s->S[0], S1 = s->S[1], S2 = s->S[2];
    int Sa = s->S[axis];
    /* transverse work-item ranges (Solver::getBoundaryRanges, Solver.cpp:412-444) */
    int n0, n1;
    if (s->dim == 1) { n0 = 1; n1 = 1; }             /* only the in-bounds item */
    else if (s->dim == 2) { n0 = axis == 0 ? S1 : S0; n1 = 1; }
    else { n0 = axis == 0 ? S1 : S0; n1 = axis == 2 ? S1 : S2; }
    for (int b = 0; b < n1; ++b)
        for (int a = 0; a < n0; ++a) {
#define AT(c) buf[offset + (long)spacing * (axis == 0 ? IDX(s, (c), a, b) : axis == 1 ? IDX(s, a, (c), b) : IDX(s, a, b, (c)))]
            if (kernel == BK_PERIODIC) {
                if (axis == 0 && (a >= S1 || b >= S2)) continue;
                if (axis == 1 && (a >= S0 || b >= S2)) continue;
                if (axis == 2 && (a >= S0 || b >= S1)) continue;
                if (minmax == 0) { AT(0) = AT(Sa - 4); AT(1) = AT(Sa - 3); }
                else { AT(Sa - 2) = AT(2); AT(Sa - 1) = AT(3); }
            } else if (kernel == BK_MIRROR) {
                if (minmax == 0) { AT(0) = AT(3); AT(1) = AT(2); }
                else { AT(Sa - 1) = AT(Sa - 4); AT(Sa - 2) = AT(Sa - 3); }
            } else if (kernel == BK_REFLECT) {
                if (minmax == 0) { AT(0) = -AT(3); AT(1) = -AT(2); }
                else { AT(Sa - 1) = -AT(Sa - 4); AT(Sa - 2) = -AT(Sa - 3); }
            } else { /* FreeFlow: a = b = c, evaluated right to left */
                if (minmax == 0) { REAL v = AT(2); AT(1) = v; AT(0) = v; }
                else { REAL v = AT(Sa - 3); AT(Sa - 2) = v; AT(Sa - 1) = v; }
            }
#undef AT
        }
}

static void FN(boundary)(FN(osolver) * s) {
    for (int i = 0; i < s->dim; ++i)
        for (int j = 0; j < s->N; ++j)
            for (int mm = 0; mm < 2; ++mm) {
                int method = s->cfg.boundary[i][mm];
                int k;
                if (method == HGPU_BOUNDARY_NONE) continue;
                else if (method == HGPU_BOUNDARY_PERIODIC) k = BK_PERIODIC;
                else if (method == HGPU_BOUNDARY_MIRROR) k = (i + 1 == j) ? BK_REFLECT : BK_MIRROR;
                else k = BK_FREEFLOW;
                FN(boundaryKernel)(s, s->state, s->N, j, k, i, mm);
            }
}

/* ---------------- Roe: calcEigenBasisSide (EulerRoe.cl:18-259), solid==0, potential==0 ---------------- */
static void FN(calcEigenBasis)(FN(osolver) * s) {
    const int N = s->N, E = N - 1, D = s->dim;
    const REAL g = s->gamma;
    FOR_CELLS(s) {
        if (!FN(inRange)(s, x, y, z, 2, 1)) continue;
        long index = IDX(s, x, y, z);
        for (int side = 0; side < D; ++side) {
            long indexPrev = index - s->step[side];
            const REAL* sL = s->state + N * indexPrev;
            const REAL* sR = s->state + N * index;
            long iface = side + D * index;
            REAL* lam = s->eigenvalues + N * iface;
            REAL* Linv = s->eigenvectors + 2 * N * N * iface;
            REAL* R = Linv + N * N;
            REAL vL[4] = {0, 0, 0, 0}, vR[4] = {0, 0, 0, 0};
            REAL rhoL = sL[0], rhoR = sR[0];
            /* VELOCITY(ptr) = (real4)(m..., 0, ...) / rho  (res/include/HydroGPU/Euler.h:6-12) */
            for (int k = 0; k < 4; ++k) vL[k] = (k < D ? sL[1 + k] : (REAL)0.f) / rhoL;
            for (int k = 0; k < 4; ++k) vR[k] = (k < D ? sR[1 + k] : (REAL)0.f) / rhoR;
            REAL invDensityL = 1.f / rhoL;                               /* :67 */
            REAL energyTotalL = sL[E] * invDensityL;
            REAL energyKineticL = .5f * DOT4(vL, vL);
            REAL energyPotentialL = s->potential[indexPrev];
            REAL energyInternalL = energyTotalL - energyKineticL - energyPotentialL;
            REAL pressureL = (g - 1.f) * rhoL * energyInternalL;
            REAL enthalpyTotalL = energyTotalL + pressureL * invDensityL;
            REAL roeWeightL = sqrt(rhoL);
            REAL invDensityR = 1.f / rhoR;                               /* :76 */
            REAL energyTotalR = sR[E] * invDensityR;
            REAL energyKineticR = .5f * DOT4(vR, vR);
            REAL energyPotentialR = s->potential[index];
            REAL energyInternalR = energyTotalR - energyKineticR - energyPotentialR;
            REAL pressureR = (g - 1.f) * rhoR * energyInternalR;
            REAL enthalpyTotalR = energyTotalR + pressureR * invDensityR;
            REAL roeWeightR = sqrt(rhoR);
            REAL norm = 1.f / (roeWeightL + roeWeightR);                /* :85 */
            REAL v[4];
            for (int k = 0; k < 4; ++k) v[k] = (roeWeightL * vL[k] + roeWeightR * vR[k]) * norm;
            REAL enthalpyTotal = (roeWeightL * enthalpyTotalL + roeWeightR * enthalpyTotalR) * norm;
            REAL energyPotential = (roeWeightL * energyPotentialL + roeWeightR * energyPotentialR) * norm;
            REAL velocitySq = DOT4(v, v);
            REAL c = sqrt((enthalpyTotal - .5f * velocitySq - energyPotential) * (g - 1.f));
            /* rotate normal velocity into x (:101-110) */
            if (side == 1) { REAL t = v[0]; v[0] = v[1]; v[1] = t; }
            else if (side == 2) { REAL t = v[0]; v[0] = v[2]; v[2] = t; }
            REAL vx = v[0], vy = v[1], vz = v[2];
            /* eigenvalues (:114-122) */
            lam[0] = vx - c;
            for (int k = 1; k < E; ++k) lam[k] = vx;
            lam[E] = vx + c;
            /* right eigenvectors, column-major [row + N*col] (:126-173) */
            R[0 + N * 0] = 1.f;
            R[1 + N * 0] = vx - c;
            if (D > 1) R[2 + N * 0] = vy;
            if (D > 2) R[3 + N * 0] = vz;
            R[E + N * 0] = enthalpyTotal - c * vx;
            R[0 + N * 1] = 1.f;
            R[1 + N * 1] = vx;
            if (D > 1) R[2 + N * 1] = vy;
            if (D > 2) R[3 + N * 1] = vz;
            R[E + N * 1] = .5f * velocitySq;
            if (D > 1) {
                R[0 + N * 2] = 0.f; R[1 + N * 2] = 0.f; R[2 + N * 2] = 1.f;
                if (D > 2) R[3 + N * 2] = 0.f;
                R[E + N * 2] = vy;
            }
            if (D > 2) {
                R[0 + N * 3] = 0.f; R[1 + N * 3] = 0.f; R[2 + N * 3] = 0.f; R[3 + N * 3] = 1.f;
                R[E + N * 3] = vz;
            }
            R[0 + N * E] = 1.f;
            R[1 + N * E] = vx + c;
            if (D > 1) R[2 + N * E] = vy;
            if (D > 2) R[3 + N * E] = vz;
            R[E + N * E] = enthalpyTotal + c * vx;
            /* left eigenvectors = inverse, [row + N*col] (:177-226) */
            REAL invDenom = .5f / (c * c);
            Linv[0 + N * 0] = (.5f * (g - 1.f) * velocitySq + c * vx) * invDenom;
            Linv[0 + N * 1] = -(c + (g - 1.f) * vx) * invDenom;
            if (D > 1) Linv[0 + N * 2] = -(g - 1.f) * vy * invDenom;
            if (D > 2) Linv[0 + N * 3] = -(g - 1.f) * vz * invDenom;
            Linv[0 + N * E] = (g - 1.f) * invDenom;
            Linv[1 + N * 0] = 1.f - (g - 1.f) * velocitySq * invDenom;
            Linv[1 + N * 1] = (g - 1.f) * vx * 2.f * invDenom;
            if (D > 1) Linv[1 + N * 2] = (g - 1.f) * vy * 2.f * invDenom;
            if (D > 2) Linv[1 + N * 3] = (g - 1.f) * vz * 2.f * invDenom;
            Linv[1 + N * E] = -(g - 1.f) * 2.f * invDenom;
            if (D > 1) {
                Linv[2 + N * 0] = -vy; Linv[2 + N * 1] = 0.f; Linv[2 + N * 2] = 1.f;
                if (D > 2) Linv[2 + N * 3] = 0.f;
                Linv[2 + N * E] = 0.f;
            }
            if (D > 2) {
                Linv[3 + N * 0] = -vz; Linv[3 + N * 1] = 0.f; Linv[3 + N * 2] = 0.f; Linv[3 + N * 3] = 1.f;
                Linv[3 + N * E] = 0.f;
            }
            Linv[E + N * 0] = (.5f * (g - 1.f) * velocitySq - c * vx) * invDenom;
            Linv[E + N * 1] = (c - (g - 1.f) * vx) * invDenom;
            if (D > 1) Linv[E + N * 2] = -(g - 1.f) * vy * invDenom;
            if (D > 2) Linv[E + N * 3] = -(g - 1.f) * vz * invDenom;
            Linv[E + N * E] = (g - 1.f) * invDenom;
            /* rotate back: swap L columns and R rows of momentum x and side (:228-255) */
            if (side > 0) {
                int a = 1, b = 1 + side;
                for (int i = 0; i < N; ++i) {
                    REAL t = Linv[i + N * a]; Linv[i + N * a] = Linv[i + N * b]; Linv[i + N * b] = t;
                    t = R[a + N * i]; R[a + N * i] = R[b + N * i]; R[b + N * i] = t;
                }
            }
        }
    }
}

/* c_i = sum_j M[i + N*j] x_j, j ascending from 0 (RoeEigenfieldLinear.cl:16-54) */
static inline void FN(matTransform)(int N, REAL* out, const REAL* M, const REAL* in) {
    for (int i = 0; i < N; ++i) {
        REAL sum = 0.f;
        for (int j = 0; j < N; ++j) sum += M[i + N * j] * in[j];
        out[i] = sum;
    }
}

/* ---------------- Roe calcCellTimestep (Roe.cl:4-65), solid==0 ---------------- */
static void FN(roeCellTimestep)(FN(osolver) * s) {
    const int N = s->N, D = s->dim;
    FOR_CELLS(s) {
        long index = IDX(s, x, y, z);
        if (!FN(inRange)(s, x, y, z, 2, 2)) {
            for (int side = 0; side < D; ++side) s->dtBuffer[side + D * index] = INFINITY;
            continue;
        }
        for (int side = 0; side < D; ++side) {
            long indexR = index + s->step[side];
            const REAL* lamL = s->eigenvalues + N * (side + D * index);
            const REAL* lamR = s->eigenvalues + N * (side + D * indexR);
            REAL maxLambda = (REAL)fmax((REAL)0., lamL[N - 1]);
            REAL minLambda = (REAL)fmin((REAL)0., lamR[0]);
            REAL dum = (REAL)(s->dx[side] / (fabs(maxLambda - minLambda) + 1e-9));
            s->dtBuffer[side + D * index] = dum;
        }
    }
}

/* ---------------- Roe calcDeltaQTilde (Roe.cl:67-168) ---------------- */
static void FN(calcDeltaQTilde)(FN(osolver) * s) {
    const int N = s->N, D = s->dim;
    FOR_CELLS(s) {
        if (!FN(inRange)(s, x, y, z, 2, 1)) continue;
        long index = IDX(s, x, y, z);
        for (int side = 0; side < D; ++side) {
            long indexPrev = index - s->step[side];
            long iface = side + D * index;
            const REAL* ev = s->eigenvectors + 2 * N * N * iface;
            REAL dS[5], dq[5];
            for (int i = 0; i < N; ++i) dS[i] = s->state[i + N * index] - s->state[i + N * indexPrev];
            FN(matTransform)(N, dq, ev, dS);
            for (int i = 0; i < N; ++i) s->deltaQTilde[N * iface + i] = dq[i];
        }
    }
}

/* ---------------- Roe calcFlux (Roe.cl:170-320) ---------------- */
static void FN(roeFlux)(FN(osolver) * s, REAL dt) {
    const int N = s->N, D = s->dim, lim = s->cfg.limiter;
    FOR_CELLS(s) {
        if (!FN(inRange)(s, x, y, z, 2, 1)) continue;
        long index = IDX(s, x, y, z);
        for (int side = 0; side < D; ++side) {
            REAL dt_dx = dt / s->dx[side];
            long indexL = index - s->step[side], indexR2 = index + s->step[side];
            long ifL = side + D * indexL, iF = side + D * index, ifR = side + D * indexR2;
            const REAL* dqL = s->deltaQTilde + N * ifL;
            const REAL* dq = s->deltaQTilde + N * iF;
            const REAL* dqR = s->deltaQTilde + N * ifR;
            const REAL* lam = s->eigenvalues + N * iF;
            const REAL* ev = s->eigenvectors + 2 * N * N * iF;
            REAL avg[5], ft[5];
            for (int i = 0; i < N; ++i) avg[i] = .5 * (s->state[i + N * index] + s->state[i + N * indexL]);
            FN(matTransform)(N, ft, ev, avg);
            for (int i = 0; i < N; ++i) {
                REAL eigenvalue = lam[i];
                ft[i] *= eigenvalue;
                REAL rTilde, theta;
                if (eigenvalue >= 0.) { rTilde = dqL[i] / dq[i]; theta = 1.; }
                else { rTilde = dqR[i] / dq[i]; theta = -1.; }
                REAL phi = FN(slopeLimiter)(lim, rTilde);
                REAL epsilon = eigenvalue * dt_dx;
                REAL deltaFluxTilde = eigenvalue * dq[i];
                ft[i] -= .5 * deltaFluxTilde * (theta + phi * (epsilon - theta));
            }
            FN(matTransform)(N, s->flux + N * iF, ev + N * N, ft);
        }
    }
}

/* ---------------- HLLC calcEigenvalues (EulerHLLC.cl:15-131) ---------------- */
static void FN(hllcEigenvalues)(FN(osolver) * s) {
    const int N = s->N, E = N - 1, D = s->dim;
    const REAL g = s->gamma;
    FOR_CELLS(s) {
        if (!FN(inRange)(s, x, y, z, 2, 1)) continue;
        long index = IDX(s, x, y, z);
        for (int side = 0; side < D; ++side) {
            long indexPrev = index - s->step[side];
            REAL sL[5], sR[5];
            for (int i = 0; i < N; ++i) { sL[i] = s->state[i + N * indexPrev]; sR[i] = s->state[i + N * index]; }
            { REAL t = sL[1]; sL[1] = sL[1 + side]; sL[1 + side] = t; t = sR[1]; sR[1] = sR[1 + side]; sR[1 + side] = t; }
            REAL* lam = s->eigenvalues + N * (side + D * index);
            REAL rhoL = sL[0];
            REAL invDensityL = 1. / rhoL;
            REAL vL[4], vR[4];
            for (int k = 0; k < 4; ++k) vL[k] = (k < D ? sL[1 + k] : (REAL)0.f) / rhoL;
            REAL velocitySqL = DOT4(vL, vL);
            REAL energyTotalL = sL[E] * invDensityL;
            REAL energyKineticL = .5f * velocitySqL;
            REAL energyPotentialL = s->potential[indexPrev];
            REAL energyInternalL = energyTotalL - energyKineticL - energyPotentialL;
            REAL pressureL = (g - 1.) * rhoL * energyInternalL;
            REAL enthalpyTotalL = energyTotalL + pressureL * invDensityL;
            REAL cL = sqrt((g - 1.) * (enthalpyTotalL - .5f * velocitySqL));
            REAL wL = sqrt(rhoL);
            REAL rhoR = sR[0];
            REAL invDensityR = 1. / rhoR;
            for (int k = 0; k < 4; ++k) vR[k] = (k < D ? sR[1 + k] : (REAL)0.f) / rhoR;
            REAL velocitySqR = DOT4(vR, vR);
            REAL energyTotalR = sR[E] * invDensityR;
            REAL energyKineticR = .5f * velocitySqR;
            REAL energyPotentialR = s->potential[index];
            REAL energyInternalR = energyTotalR - energyKineticR - energyPotentialR;
            REAL pressureR = (g - 1.) * rhoR * energyInternalR;
            REAL enthalpyTotalR = energyTotalR + pressureR * invDensityR;
            REAL cR = sqrt((g - 1.) * (enthalpyTotalR - .5f * velocitySqR));
            REAL wR = sqrt(rhoR);
            REAL norm = 1. / (wL + wR);
            REAL vx = (wL * vL[0] + wR * vR[0]) * norm;
            REAL pStar = (REAL)fmax(0., .5f * (pressureL + pressureR) - .5f * (vR[0] - vL[0]) * .5f * (rhoL + rhoR) * .5f * (cL + cR));
            REAL qL = pStar <= pressureL ? 1. : sqrt(1. + (g + 1.) / (2. * g) * (pStar / pressureL - 1.));
            REAL qR = pStar <= pressureR ? 1. : sqrt(1. + (g + 1.) / (2. * g) * (pStar / pressureR - 1.));
            REAL sl = vL[0] - cL * qL;
            REAL sr = vR[0] + cR * qR;
            lam[0] = sl;
            for (int k = 1; k < E; ++k) lam[k] = vx;
            lam[E] = sr;
        }
    }
}

/* ---------------- HLLC calcCellTimestep (EulerHLLC.cl:135-168) ---------------- */
static void FN(hllcCellTimestep)(FN(osolver) * s) {
    const int N = s->N, E = N - 1, D = s->dim;
    FOR_CELLS(s) {
        long index = IDX(s, x, y, z);
        if (!FN(inRange)(s, x, y, z, 2, 1)) { s->dtBuffer[index] = INFINITY; continue; }
        REAL result = INFINITY;
        for (int side = 0; side < D; ++side) {
            long indexNext = index + s->step[side];
            const REAL* lamL = s->eigenvalues + N * (side + D * index);
            const REAL* lamR = s->eigenvalues + N * (side + D * indexNext);
            REAL minLambda = (REAL)fmin(0., lamR[0]);
            REAL maxLambda = (REAL)fmax(0., lamL[E]);
            REAL dum = s->dx[side] / (maxLambda - minLambda);
            result = (REAL)fmin(result, dum);
        }
        s->dtBuffer[index] = result;
    }
}

/* ---------------- HLLC calcFlux (EulerHLLC.cl:170-445), HLLC_METHOD 2, no limiter ---------------- */
static void FN(hllcFlux)(FN(osolver) * s) {
    const int N = s->N, E = N - 1, D = s->dim;
    const REAL g = s->gamma;
    FOR_CELLS(s) {
        if (!FN(inRange)(s, x, y, z, 2, 1)) continue;
        long index = IDX(s, x, y, z);
        for (int side = 0; side < D; ++side) {
            long indexPrev = index - s->step[side];
            long iF = side + D * index;
            REAL sL[5], sR[5];
            for (int i = 0; i < N; ++i) { sL[i] = s->state[i + N * indexPrev]; sR[i] = s->state[i + N * index]; }
            { REAL t = sL[1]; sL[1] = sL[1 + side]; sL[1 + side] = t; t = sR[1]; sR[1] = sR[1 + side]; sR[1 + side] = t; }
            const REAL* lam = s->eigenvalues + N * iF;
            REAL* flux = s->flux + N * iF;
            REAL rhoL = sL[0];
            REAL invDensityL = 1. / rhoL;
            REAL vL[4], vR[4];
            for (int k = 0; k < 4; ++k) vL[k] = (k < D ? sL[1 + k] : (REAL)0.f) / rhoL;
            REAL velocitySqL = DOT4(vL, vL);
            REAL energyTotalL = sL[E] * invDensityL;
            REAL energyKineticL = .5f * velocitySqL;
            REAL energyPotentialL = s->potential[indexPrev];
            REAL energyInternalL = energyTotalL - energyKineticL - energyPotentialL;
            REAL pressureL = (g - 1.) * rhoL * energyInternalL;
            REAL enthalpyTotalL = energyTotalL + pressureL * invDensityL;
            REAL rhoR = sR[0];
            REAL invDensityR = 1. / rhoR;
            for (int k = 0; k < 4; ++k) vR[k] = (k < D ? sR[1 + k] : (REAL)0.f) / rhoR;
            REAL velocitySqR = DOT4(vR, vR);
            REAL energyTotalR = sR[E] * invDensityR;
            REAL energyKineticR = .5f * velocitySqR;
            REAL energyPotentialR = s->potential[index];
            REAL energyInternalR = energyTotalR - energyKineticR - energyPotentialR;
            REAL pressureR = (g - 1.) * rhoR * energyInternalR;
            REAL enthalpyTotalR = energyTotalR + pressureR * invDensityR;
            REAL sl = lam[0], sr = lam[E];
            REAL fL[5], fR[5];
            fL[0] = rhoL * vL[0];
            fL[1] = rhoL * vL[0] * vL[0] + pressureL;
            if (D > 1) fL[2] = rhoL * vL[1] * vL[0];
            if (D > 2) fL[3] = rhoL * vL[2] * vL[0];
            fL[E] = rhoL * enthalpyTotalL * vL[0];
            fR[0] = rhoR * vR[0];
            fR[1] = rhoR * vR[0] * vR[0] + pressureR;
            if (D > 1) fR[2] = rhoR * vR[1] * vR[0];
            if (D > 2) fR[3] = rhoR * vR[2] * vR[0];
            fR[E] = rhoR * enthalpyTotalR * vR[0];
            REAL sStar = (rhoR * vR[0] * (sr - vR[0]) - rhoL * vL[0] * (sl - vL[0]) + pressureL - pressureR)
                         / (rhoR * (sr - vR[0]) - rhoL * (sl - vL[0]));
            if (0. <= sl) {
                for (int i = 0; i < N; ++i) flux[i] = fL[i];
            } else if (sl <= 0. && 0. <= sStar) {
                REAL pLR = .5f * (pressureL + pressureR + rhoL * (sl - vL[0]) * (sStar - vL[0]) + rhoR * (sr - vR[0]) * (sStar - vR[0]));
                flux[0] = sStar * (sl * sL[0] - fL[0]) / (sl - sStar);
                flux[1] = (sStar * (sl * sL[1] - fL[1]) + sl * pLR) / (sl - sStar);
                if (D > 1) flux[2] = sStar * (sl * sL[2] - fL[2]) / (sl - sStar);
                if (D > 2) flux[3] = sStar * (sl * sL[3] - fL[3]) / (sl - sStar);
                flux[E] = (sStar * (sl * sL[E] - fL[E]) + sl * pLR * sStar) / (sl - sStar);
            } else if (sStar <= 0. && 0. <= sr) {
                REAL pLR = .5f * (pressureL + pressureR + rhoL * (sl - vL[0]) * (sStar - vL[0]) + rhoR * (sr - vR[0]) * (sStar - vR[0]));
                flux[0] = sStar * (sr * sR[0] - fR[0]) / (sr - sStar);
                flux[1] = (sStar * (sr * sR[1] - fR[1]) + sr * pLR) / (sr - sStar);
                if (D > 1) flux[2] = sStar * (sr * sR[2] - fR[2]) / (sr - sStar);
                if (D > 2) flux[3] = sStar * (sr * sR[3] - fR[3]) / (sr - sStar);
                flux[E] = (sStar * (sr * sR[E] - fR[E]) + sr * pLR * sStar) / (sr - sStar);
            } else if (sr <= 0.) {
                for (int i = 0; i < N; ++i) flux[i] = fR[i];
            }
            /* no branch taken: the buffer keeps its previous flux (stale), and is still rotated back */
            { REAL t = flux[1]; flux[1] = flux[1 + side]; flux[1 + side] = t; }
        }
    }
}

/* ---------------- EulerHLL calcEigenvalues (EulerHLL.cl:17-138) ----------------
 * Davis direct bounded wave speeds: sl = min(vL - cL, v - c), sr = max(vR + cR, v + c)
 * with v, c from the Roe averages.  `.5 * velocitySq` and `(gamma - 1.)` are double
 * literals here (EulerHLLC.cl writes `.5f`): FP32 evaluates them in double. */
static void FN(hllEigenvalues)(FN(osolver) * s) {
    const int N = s->N, E = N - 1, D = s->dim;
    const REAL g = s->gamma;
    FOR_CELLS(s) {
        if (!FN(inRange)(s, x, y, z, 2, 1)) continue;
        long index = IDX(s, x, y, z);
        for (int side = 0; side < D; ++side) {
            long indexPrev = index - s->step[side];
            REAL sL[5], sR[5];
            for (int i = 0; i < N; ++i) { sL[i] = s->state[i + N * indexPrev]; sR[i] = s->state[i + N * index]; }
            { REAL t = sL[1]; sL[1] = sL[1 + side]; sL[1 + side] = t; t = sR[1]; sR[1] = sR[1 + side]; sR[1 + side] = t; }
            REAL* lam = s->eigenvalues + N * (side + D * index);
            REAL rhoL = sL[0];
            REAL invDensityL = 1. / rhoL;
            REAL vL[4], vR[4];
            for (int k = 0; k < 4; ++k) vL[k] = (k < D ? sL[1 + k] : (REAL)0.f) / rhoL;
            REAL velocitySqL = DOT4(vL, vL);
            REAL energyTotalL = sL[E] * invDensityL;
            REAL energyKineticL = .5 * velocitySqL;
            REAL energyPotentialL = s->potential[indexPrev];
            REAL energyInternalL = energyTotalL - energyKineticL - energyPotentialL;
            REAL pressureL = (g - 1.) * rhoL * energyInternalL;
            REAL enthalpyTotalL = energyTotalL + pressureL * invDensityL;
            REAL speedOfSoundL = sqrt((g - 1.) * (enthalpyTotalL - .5 * velocitySqL));
            REAL roeWeightL = sqrt(rhoL);
            REAL rhoR = sR[0];
            REAL invDensityR = 1. / rhoR;
            for (int k = 0; k < 4; ++k) vR[k] = (k < D ? sR[1 + k] : (REAL)0.f) / rhoR;
            REAL velocitySqR = DOT4(vR, vR);
            REAL energyTotalR = sR[E] * invDensityR;
            REAL energyKineticR = .5 * velocitySqR;
            REAL energyPotentialR = s->potential[index];
            REAL energyInternalR = energyTotalR - energyKineticR - energyPotentialR;
            REAL pressureR = (g - 1.) * rhoR * energyInternalR;
            REAL enthalpyTotalR = energyTotalR + pressureR * invDensityR;
            REAL speedOfSoundR = sqrt((g - 1.) * (enthalpyTotalR - .5 * velocitySqR));
            REAL roeWeightR = sqrt(rhoR);
            REAL norm = 1. / (roeWeightL + roeWeightR);
            REAL v[4];
            for (int k = 0; k < 4; ++k) v[k] = (roeWeightL * vL[k] + roeWeightR * vR[k]) * norm;
            REAL enthalpyTotal = (roeWeightL * enthalpyTotalL + roeWeightR * enthalpyTotalR) * norm;
            REAL energyPotential = (roeWeightL * energyPotentialL + roeWeightR * energyPotentialR) * norm;
            REAL velocitySq = DOT4(v, v);
            REAL speedOfSound = sqrt((g - 1.) * (enthalpyTotal - .5 * velocitySq - energyPotential));
            REAL eigenvaluesMinL = vL[0] - speedOfSoundL;
            REAL eigenvaluesMaxR = vR[0] + speedOfSoundR;
            REAL eigenvaluesMin = v[0] - speedOfSound;
            REAL eigenvaluesMax = v[0] + speedOfSound;
            lam[0] = (REAL)fmin(eigenvaluesMinL, eigenvaluesMin);
            for (int k = 1; k < E; ++k) lam[k] = v[0];
            lam[E] = (REAL)fmax(eigenvaluesMaxR, eigenvaluesMax);
        }
    }
}

/* ---------------- EulerHLL calcFlux (EulerHLL.cl:185-346): the two-state HLL flux ---------------- */
static void FN(hllFlux)(FN(osolver) * s) {
    const int N = s->N, E = N - 1, D = s->dim;
    const REAL g = s->gamma;
    FOR_CELLS(s) {
        if (!FN(inRange)(s, x, y, z, 2, 1)) continue;
        long index = IDX(s, x, y, z);
        for (int side = 0; side < D; ++side) {
            long indexPrev = index - s->step[side];
            long iF = side + D * index;
            REAL sL[5], sR[5];
            for (int i = 0; i < N; ++i) { sL[i] = s->state[i + N * indexPrev]; sR[i] = s->state[i + N * index]; }
            { REAL t = sL[1]; sL[1] = sL[1 + side]; sL[1 + side] = t; t = sR[1]; sR[1] = sR[1 + side]; sR[1 + side] = t; }
            const REAL* lam = s->eigenvalues + N * iF;
            REAL* flux = s->flux + N * iF;
            REAL rhoL = sL[0];
            REAL invDensityL = 1. / rhoL;
            REAL vL[4], vR[4];
            for (int k = 0; k < 4; ++k) vL[k] = (k < D ? sL[1 + k] : (REAL)0.f) / rhoL;
            REAL velocitySqL = DOT4(vL, vL);
            REAL energyTotalL = sL[E] * invDensityL;
            REAL energyKineticL = .5 * velocitySqL;
            REAL energyPotentialL = s->potential[indexPrev];
            REAL energyInternalL = energyTotalL - energyKineticL - energyPotentialL;
            REAL pressureL = (g - 1.) * rhoL * energyInternalL;
            REAL enthalpyTotalL = energyTotalL + pressureL * invDensityL;
            REAL rhoR = sR[0];
            REAL invDensityR = 1. / rhoR;
            for (int k = 0; k < 4; ++k) vR[k] = (k < D ? sR[1 + k] : (REAL)0.f) / rhoR;
            REAL velocitySqR = DOT4(vR, vR);
            REAL energyTotalR = sR[E] * invDensityR;
            REAL energyKineticR = .5 * velocitySqR;
            REAL energyPotentialR = s->potential[index];
            REAL energyInternalR = energyTotalR - energyKineticR - energyPotentialR;
            REAL pressureR = (g - 1.) * rhoR * energyInternalR;
            REAL enthalpyTotalR = energyTotalR + pressureR * invDensityR;
            REAL sl = lam[0], sr = lam[N - 1];
            REAL fL[5], fR[5];
            fL[0] = rhoL * vL[0];
            fL[1] = rhoL * vL[0] * vL[0] + pressureL;
            if (D > 1) fL[2] = rhoL * vL[1] * vL[0];
            if (D > 2) fL[3] = rhoL * vL[2] * vL[0];
            fL[E] = rhoL * enthalpyTotalL * vL[0];
            fR[0] = rhoR * vR[0];
            fR[1] = rhoR * vR[0] * vR[0] + pressureR;
            if (D > 1) fR[2] = rhoR * vR[1] * vR[0];
            if (D > 2) fR[3] = rhoR * vR[2] * vR[0];
            fR[E] = rhoR * enthalpyTotalR * vR[0];
            if (0. <= sl) {
                for (int i = 0; i < N; ++i) flux[i] = fL[i];
            } else if (sl <= 0. && 0. <= sr) {
                REAL invDenom = 1. / (sr - sl);
                for (int i = 0; i < N; ++i) flux[i] = (sr * fL[i] - sl * fR[i] + sl * sr * (sR[i] - sL[i])) * invDenom;
            } else if (sr <= 0.) {
                for (int i = 0; i < N; ++i) flux[i] = fR[i];
            }
            /* no branch taken: the buffer keeps its previous flux (stale), and is still rotated back */
            { REAL t = flux[1]; flux[1] = flux[1 + side]; flux[1 + side] = t; }
        }
    }
}

/* ---------------- convertToTex (EulerMHDCommon.cl:4-116): the display scalar ----------------
 * `method` is the reference's DISPLAY_* index, whose numbering depends on dim
 * (Euler.cpp:18-27): DENSITY, VELOCITY, VELOCITY_X, [VELOCITY_Y], [VELOCITY_Z],
 * PRESSURE, ENERGY_INTERNAL, ENERGY_KINETIC, ENERGY_TOTAL, POTENTIAL.  Every cell,
 * ghosts included; the float4's x component. */
static int FN(display)(FN(osolver) * s, int method, float* out) {
    const int N = s->N, E = N - 1, D = s->dim;
    const REAL g = s->gamma;
    int kind = method;                       /* 0..9 in the dim-3 numbering */
    if (method < 0 || method >= 7 + D) return HGPU_ERR_ARG;
    if (method >= 2 + D) kind = method + (3 - D);
    FOR_CELLS(s) {
        long index = IDX(s, x, y, z);
        const REAL* st = s->state + N * index;
        REAL density = st[0];
        REAL v[4];
        for (int k = 0; k < 4; ++k) v[k] = (k < D ? st[1 + k] : (REAL)0.f) / density;
        REAL energyTotal = st[E];
        REAL velocitySq = DOT4(v, v);
        REAL energyKinetic = .5 * density * velocitySq;
        REAL energyPotential = density * s->potential[index];
        REAL energyInternal = energyTotal - energyKinetic - energyPotential;
        REAL value = 0;
        switch (kind) {
        case 0: value = density; break;
        case 1: value = sqrt(velocitySq); break;
        case 2: value = v[0]; break;
        case 3: value = v[1]; break;
        case 4: value = v[2]; break;
        case 5: value = (g - 1.) * energyInternal; break;
        case 6: value = energyInternal; break;
        case 7: value = energyKinetic; break;
        case 8: value = energyTotal; break;
        case 9: value = s->potential[index]; break;
        }
        out[index] = (float)value;
    }
    return HGPU_OK;
}

/* ---------------- calcFluxDeriv (CalcFluxDeriv.cl:7-44) ---------------- */
static void FN(calcFluxDeriv)(FN(osolver) * s, REAL* deriv) {
    const int N = s->N, D = s->dim;
    FOR_CELLS(s) {
        if (!FN(inRange)(s, x, y, z, 2, 2)) continue;
        long index = IDX(s, x, y, z);
        REAL* d = deriv + N * index;
        for (int side = 0; side < D; ++side) {
            long iF = side + D * index;
            long iFn = iF + D * s->step[side];
            for (int j = 0; j < N; ++j) {
                REAL deltaFlux = s->flux[N * iFn + j] - s->flux[N * iF + j];
                d[j] -= deltaFlux / s->dx[side];
            }
        }
    }
}

/* ---------------- self-gravity: SelfGravitation.cpp:35-140, SelfGravitation.cl:20-102 ---------------- */

/* potentialBoundary (SelfGravitation.cpp:126-140): each axis, min then max, with the
 * potential's kernel for the method (SelfGravitationBehavior.h:22-34: PERIODIC ->
 * periodic, MIRROR and FREEFLOW -> free flow) on the stride-1 potential buffer */
static void FN(potentialBoundary)(FN(osolver) * s) {
    for (int i = 0; i < s->dim; ++i)
        for (int mm = 0; mm < 2; ++mm) {
            int method = s->cfg.boundary[i][mm];
            if (method == HGPU_BOUNDARY_NONE) continue;
            FN(boundaryKernel)(s, s->potential, 1, 0, method == HGPU_BOUNDARY_PERIODIC ? BK_PERIODIC : BK_FREEFLOW,
                               i, mm);
        }
}

/* gravityPotentialPoissonRelax (SelfGravitation.cl:20-63) at one interior cell */
static void FN(poissonRelaxCell)(FN(osolver) * s, int x, int y, int z) {
    const int D = s->dim;
    REAL* phi = s->potential;
    long index = IDX(s, x, y, z);
    REAL skewSum = 0.;
    if (x < s->S[0] - 3) skewSum += phi[index + s->step[0]] / (s->dx[0] * s->dx[0]);
    if (x > 2) skewSum += phi[index - s->step[0]] / (s->dx[0] * s->dx[0]);
    if (D > 1) {
        if (y < s->S[1] - 3) skewSum += phi[index + s->step[1]] / (s->dx[1] * s->dx[1]);
        if (y > 2) skewSum += phi[index - s->step[1]] / (s->dx[1] * s->dx[1]);
    }
    if (D > 2) {
        if (z < s->S[2] - 3) skewSum += phi[index + s->step[2]] / (s->dx[2] * s->dx[2]);
        if (z > 2) skewSum += phi[index - s->step[2]] / (s->dx[2] * s->dx[2]);
    }
    REAL diag;
    if (D == 1) diag = -2. * (1. / (s->dx[0] * s->dx[0]));
    else if (D == 2) diag = -2. * (1. / (s->dx[0] * s->dx[0]) + 1. / (s->dx[1] * s->dx[1]));
    else diag = -2. * (1. / (s->dx[0] * s->dx[0]) + 1. / (s->dx[1] * s->dx[1]) + 1. / (s->dx[2] * s->dx[2]));
    const REAL G = s->G;
    REAL density = s->state[s->N * index];
    phi[index] = (4. * M_PI * G * density - skewSum) / diag;
}

/* One relaxation launch.  The reference kernel writes the potential in place while
 * other work-items read it, so its result depends on the order the device runs the
 * work-items in; this restates the red-black order: every interior cell with
 * x + y + z even, then every odd one (cells of one parity never read each other). */
static void FN(poissonRelax)(FN(osolver) * s) {
    for (int colour = 0; colour < 2; ++colour) {
        FOR_CELLS(s) {
            if (((x + y + z) & 1) != colour) continue;
            if (!FN(inRange)(s, x, y, z, 2, 2)) continue;
            FN(poissonRelaxCell)(s, x, y, z);
        }
    }
}

/* sweeps x (potentialBoundary, relax): SelfGravitation.cpp:81-86 and :112-117 */
static void FN(relaxPotential)(FN(osolver) * s, int sweeps) {
    for (int i = 0; i < sweeps; ++i) {
        FN(potentialBoundary)(s);
        FN(poissonRelax)(s);
    }
}

/* SelfGravitation::resetState (SelfGravitation.cpp:35-98) after the state upload:
 * potentialVec = -density with useGravity, else the initial conditions' channel (pot,
 * NULL = zero); upload it; relax 100 x gaussSeidelMaxIter times with useGravity; add
 * potentialVec (the host vector, not the relaxed buffer) to the total energy. */
static void FN(resetPotential)(FN(osolver) * s, const REAL* pot) {
    const int N = s->N, E = N - 1;
    REAL* vec = (REAL*)calloc((size_t)s->V, sizeof(REAL));
    for (long i = 0; i < s->V; ++i)
        vec[i] = s->cfg.use_gravity ? -s->state[N * i] : (pot ? pot[i] : (REAL)0);
    memcpy(s->potential, vec, sizeof(REAL) * (size_t)s->V);
    if (s->cfg.use_gravity)
        for (int tries = 0; tries < 100; ++tries) FN(relaxPotential)(s, s->cfg.gauss_seidel_max_iter);
    for (long i = 0; i < s->V; ++i) s->state[E + N * i] += vec[i];
    free(vec);
}

/* ---------------- calcGravityDeriv (SelfGravitation.cl:65-102) ---------------- */
static void FN(calcGravityDeriv)(FN(osolver) * s, REAL* deriv) {
    const int N = s->N, D = s->dim, E = N - 1;
    FOR_CELLS(s) {
        if (!FN(inRange)(s, x, y, z, 2, 2)) continue;
        long index = IDX(s, x, y, z);
        REAL* d = deriv + N * index;
        const REAL* st = s->state + N * index;
        REAL density = st[0];
        REAL derivEnergyTotal = 0.;
        for (int side = 0; side < D; ++side) {
            long ip = index - s->step[side], in = index + s->step[side];
            REAL gradient = (s->potential[in] - s->potential[ip]) / (2. * s->dx[side]);
            REAL gravity = -gradient;
            d[side + 1] -= density * gravity;
            derivEnergyTotal -= density * gravity * st[side + 1];
        }
        d[E] += derivEnergyTotal;
    }
}

/* ---------------- integrators ---------------- */
static void FN(multAdd)(FN(osolver) * s, REAL* result, const REAL* b, REAL c) {  /* Common.cl:201-210 */
    long n = s->V * s->N;
    _Pragma("omp parallel for schedule(static)")
    for (long i = 0; i < n; ++i) result[i] = result[i] + b[i] * c;
}

static void FN(callback)(FN(osolver) * s, int kind, REAL* deriv, REAL dt) {
    if (kind == CB_FLUX) {
        if (!s->isHLLC) {              /* Roe::calcDeriv (Roe.cpp:101-112) */
            FN(calcDeltaQTilde)(s);
            FN(roeFlux)(s, dt);
        } else {                       /* HLL::step callback (HLL.cpp:40-47) */
            if (s->isHLL) FN(hllFlux)(s);
            else FN(hllcFlux)(s);
        }
        FN(calcFluxDeriv)(s, deriv);
    } else {                           /* SelfGravitation::applyPotential (SelfGravitation.cpp:100-124) */
        if (s->cfg.use_gravity) FN(relaxPotential)(s, s->cfg.gauss_seidel_max_iter);
        FN(calcGravityDeriv)(s, deriv);
        FN(boundary)(s);
    }
}

static void FN(integrate)(FN(osolver) * s, REAL dt, int kind) {
    size_t bytes = sizeof(REAL) * (size_t)s->V * s->N;
    if (s->cfg.integrator == HGPU_INTEGRATOR_FORWARD_EULER) {   /* ForwardEuler.cpp:20-32 */
        memset(s->db[0], 0, bytes);
        FN(callback)(s, kind, s->db[0], dt);
        FN(multAdd)(s, s->state, s->db[0], dt);
        return;
    }
    REAL A[4][4], B[4][4];                                       /* RungeKutta.h:59-125 */
    int order = FN(tableau)(s->cfg.integrator, A, B);
    int need;
    need = 0; for (int m = 0; m < order; ++m) need |= A[m][0] != 0;
    if (need) memcpy(s->sb[0], s->state, bytes);
    need = 0; for (int m = 0; m < order; ++m) need |= B[m][0] != 0;
    if (need) { memset(s->db[0], 0, bytes); FN(callback)(s, kind, s->db[0], dt); }
    for (int i = 1; i <= order; ++i) {
        memset(s->state, 0, bytes);
        for (int k = 0; k < i; ++k) {
            if (A[i - 1][k] != 0) FN(multAdd)(s, s->state, s->sb[k], A[i - 1][k]);
            if (B[i - 1][k] != 0) FN(multAdd)(s, s->state, s->db[k], (REAL)(B[i - 1][k] * dt));
        }
        if (i < order) {
            need = 0; for (int m = i; m < order; ++m) need |= A[m][i] != 0;
            if (need) memcpy(s->sb[i], s->state, bytes);
            need = 0; for (int m = i; m < order; ++m) need |= B[m][i] != 0;
            if (need) { memset(s->db[i], 0, bytes); FN(callback)(s, kind, s->db[i], dt); }
        }
    }
}

/* findMinTimestep (Solver.cpp:466-516, Common.cl:9-40): min over dtBuffer, then * cfl.
 * The reference's 16-ary tree gives the same minimum for any order unless a NaN is
 * present; here a NaN is reported through *nonfinite. */
static REAL FN(findMinTimestep)(FN(osolver) * s, int* nonfinite) {
    long n = s->V * s->dim;
    REAL acc = INFINITY;
    int bad = 0;
    for (long i = 0; i < n; ++i) {
        REAL e = s->dtBuffer[i];
        if (e != e) bad = 1;
        acc = (acc < e) ? acc : e;
    }
    if (nonfinite) *nonfinite = bad;
    return (REAL)(acc * s->cfl);
}

static int FN(update)(FN(osolver) * s, int* nonfinite) {   /* Solver::update (Solver.cpp:521-546) */
    FN(boundary)(s);
    if (s->isHLLC) {                                         /* HLL::initStep (HLL.cpp:31-33) */
        if (s->isHLL) FN(hllEigenvalues)(s);
        else FN(hllcEigenvalues)(s);
    }
    REAL dt;
    if (s->cfg.use_fixed_dt) dt = (REAL)s->cfg.fixed_dt;
    else if (!s->isHLLC) {                                   /* Roe::calcTimestep (Roe.cpp:88-92) */
        FN(calcEigenBasis)(s);
        FN(roeCellTimestep)(s);
        dt = FN(findMinTimestep)(s, nonfinite);
    } else {                                                 /* HLL::calcTimestep (HLL.cpp:35-38) */
        FN(hllcCellTimestep)(s);
        dt = FN(findMinTimestep)(s, nonfinite);
    }
    s->lastDtReal = dt;
    s->lastDt = (double)dt;
    FN(integrate)(s, dt, CB_FLUX);                           /* Roe::step / HLL::step */
    FN(integrate)(s, dt, CB_GRAVITY);                        /* selfgrav->applyPotential(dt) */
    return 0;
}

static void FN(destroy)(FN(osolver) * s) {
    if (!s) return;
    free(s->state); free(s->potential); free(s->eigenvalues); free(s->eigenvectors);
    free(s->deltaQTilde); free(s->flux); free(s->dtBuffer);
    for (int i = 0; i < 4; ++i) { free(s->sb[i]); free(s->db[i]); }
    free(s);
}

static FN(osolver) * FN(create)(const hgpu_config* cfg, int dim, const double dxBaked[3], double gammaBaked,
                               double gBaked) {
    FN(osolver)* s = (FN(osolver)*)calloc(1, sizeof(FN(osolver)));
    s->cfg = *cfg;
    s->dim = dim;
    s->N = dim + 2;
    for (int i = 0; i < 3; ++i) { s->S[i] = cfg->size[i]; s->dx[i] = (REAL)dxBaked[i]; }
    s->step[0] = 1; s->step[1] = s->S[0]; s->step[2] = s->S[0] * s->S[1];
    s->V = (long)s->S[0] * s->S[1] * s->S[2];
    s->gamma = (REAL)gammaBaked;
    s->G = (REAL)gBaked;
    s->cfl = cfg->cfl;
    s->isHLLC = cfg->solver == HGPU_SOLVER_HLLC || cfg->solver == HGPU_SOLVER_HLL;
    s->isHLL = cfg->solver == HGPU_SOLVER_HLL;
    size_t vn = (size_t)s->V * s->N;
    s->state = (REAL*)calloc(vn, sizeof(REAL));
    s->potential = (REAL*)calloc((size_t)s->V, sizeof(REAL));
    s->eigenvalues = (REAL*)calloc(vn * dim, sizeof(REAL));
    if (!s->isHLLC) {
        s->eigenvectors = (REAL*)calloc(vn * dim * 2 * s->N, sizeof(REAL));
        s->deltaQTilde = (REAL*)calloc(vn * dim, sizeof(REAL));
    }
    s->flux = (REAL*)calloc(vn * dim, sizeof(REAL));
    s->dtBuffer = (REAL*)malloc(sizeof(REAL) * (size_t)s->V * dim);
    for (long i = 0; i < s->V * dim; ++i) s->dtBuffer[i] = REAL_MAX;
    for (int i = 0; i < 4; ++i) {
        s->sb[i] = (REAL*)calloc(vn, sizeof(REAL));
        s->db[i] = (REAL*)calloc(vn, sizeof(REAL));
    }
    return s;
}
