/*
 * ORACLE — test infrastructure only. Nothing in the product links or calls
 * this file; only tests/, the smoke check and bench.py's CPU-baseline leg do,
 * and only as the checker or the timed CPU baseline.
 *
 * A plain-C restatement of torchsim's real-subspace extended-phase-graph
 * (EPG) state machine over the reference's packed event buffers. It is
 * compiled twice from this one source:
 *
 *   REAL=double  the FP64 oracle every CUDA result is judged against;
 *   REAL=float   an FP32 port that keeps the reference's statement order so
 *                that, built with -ffp-contract=off like the reference
 *                (CMakeLists.txt:48-53), it reproduces the reference's own CPU
 *                kernel; it is the "port" CPU baseline where the reference
 *                cannot be built (the GPU host).
 *
 * What each function follows in the reference (src/torchsim/_epg_cpu.cpp):
 *   shift                 shift_real                       3010-3027
 *   shift_adjoint         shift_real_adjoint               5950-5971
 *   run_forward           simulate_real_range              3041-3128
 *   run_tangent           simulate_real_jvp_range          3136-3285
 *   run_tangent_lanes     simulate_real_jvp_atom_lane_range 3503-3695
 *   run_adjoint           simulate_real_vjp_range          5985-6232
 *   run_second            simulate_real_vjp_jvp_range      7028-7330
 *                         (dual arithmetic 346-365, 407-418, 768-775, 6964-6967)
 *   run_forward_complex   simulate_range<INSTANT, ONE>     4216-4566
 *                         with shift 2164-2174, rotate 2176-2208
 *   run_adjoint_complex   simulate_vjp_range<INSTANT, ONE> 4840-5985
 * Action bits are the packed action word (_epg_cpu.cpp:36-41,
 * sequence/_accelerators.py:77-84). Event kinds: 0 wait, 1 RF, 2 ADC
 * (sequence/_description.py:31-36). The work range enumerates (train, atom)
 * train-major and the output row of a work item is (train*atoms+atom)
 * (_epg_cpu.cpp:278-296).
 *
 * The complex forward covers what leaves the real subspace on one pool with
 * instant RF: RF and receiver phases, a transmit phase (B1phase) and
 * off-resonance (B0) per voxel. Complex products are written out as
 * std::complex<float> evaluates them (re = ac - bd, im = ad + bc, each
 * product rounded, no contraction), so the FP32 port reproduces the
 * reference's complex kernel too.
 *
 * Out of scope: diffusion damping, flow, pools, shaped/dynamic RF. Null
 * tissue pointers stand for the identity value (m0 = b1 = inversion
 * efficiency = 1, B1phase = B0 = 0), as the reference's feature mask does.
 */
#include <math.h>
#include <pthread.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#ifndef REAL
#define REAL double
#endif
#ifndef SUFFIX
#define SUFFIX f64
#endif
#define GLUE2(a, b) a##_##b
#define GLUE(a, b) GLUE2(a, b)
#define NAME(x) GLUE(x, SUFFIX)

#if defined(REAL_IS_FLOAT)
#define EXP expf
#define COS cosf
#define SIN sinf
#define LIT(x) x##F
#else
#define EXP exp
#define COS cos
#define SIN sin
#define LIT(x) x
#endif

enum {
    A_PRE_SHIFT = 1,
    A_POST_SHIFT = 2,
    A_INVERSION = 4,
    A_SPOIL_AFTER = 8,
    A_SHIFT_AFTER = 16,
    A_RECORD = 32,
};

/* The inputs one run reads. Tissue arrays have atom_count entries; duration
 * and flip have train_count*event_count; kind, action and output_index have
 * event_count. */
typedef struct {
    const float* t1_ms;
    const float* t2_ms;
    const float* m0;         /* nullable: 1 */
    const float* b1;         /* nullable: 1 */
    const float* inversion;  /* nullable: 1 */
    const float* duration_s;
    const int32_t* kind;
    const float* flip_rad;
    const uint8_t* action;
    const int32_t* output_index;
    int64_t atom_count;
    int64_t train_count;
    int64_t event_count;
    int64_t state_count;
    int64_t output_count;
} oracle_case;

/* One forward-mode direction: each pointer nullable (zero direction). */
typedef struct {
    const float* t1_ms;
    const float* t2_ms;
    const float* m0;
    const float* b1;
    const float* inversion;
    const float* duration_s;
    const float* flip_rad;
} oracle_direction;

static inline REAL tissue(const float* p, int64_t atom, REAL identity) {
    return p ? (REAL)p[atom] : identity;
}

/* F+ takes order k-1, F- takes order k+1, the top F- order is lost and
 * F+[0] is the conjugate of the new F-[0], which in the real subspace is its
 * negative (_epg_cpu.cpp:3010-3027). */
static void shift(REAL* plus, REAL* minus, int64_t states) {
    for (int64_t s = 0; s + 1 < states; ++s) minus[s] = minus[s + 1];
    minus[states - 1] = LIT(0.0);
    for (int64_t s = states - 1; s > 0; --s) plus[s] = plus[s - 1];
    plus[0] = -minus[0];
}

/* Transpose of shift (_epg_cpu.cpp:5950-5971). */
static void shift_adjoint(REAL* plus_bar, REAL* minus_bar, int64_t states) {
    const REAL carry = -plus_bar[0];
    for (int64_t s = 0; s + 1 < states; ++s) plus_bar[s] = plus_bar[s + 1];
    plus_bar[states - 1] = LIT(0.0);
    for (int64_t s = states - 1; s > 0; --s) minus_bar[s] = minus_bar[s - 1];
    minus_bar[0] = LIT(0.0);
    if (states > 1) minus_bar[1] += carry;
}

/* Forward over work items [begin, end). Output planes as the reference's:
 * real plane written 0, imaginary plane m0*F+[0]. */
static void run_forward(const oracle_case* c, int64_t begin, int64_t end,
                        REAL* out_real, REAL* out_imag) {
    const int64_t S = c->state_count;
    REAL* plus = (REAL*)calloc((size_t)(3 * S), sizeof(REAL));
    REAL* minus = plus + S;
    REAL* lon = minus + S;
    for (int64_t work = begin; work < end; ++work) {
        const int64_t train = work / c->atom_count;
        const int64_t atom = work % c->atom_count;
        const float* duration = c->duration_s + train * c->event_count;
        const float* flip = c->flip_rad + train * c->event_count;
        const int64_t out_base = (train * c->atom_count + atom) * c->output_count;
        memset(plus, 0, sizeof(REAL) * (size_t)(3 * S));
        lon[0] = LIT(1.0);
        const REAL r1 = LIT(1000.0) / (REAL)c->t1_ms[atom];
        const REAL r2 = LIT(1000.0) / (REAL)c->t2_ms[atom];
        const REAL b1 = tissue(c->b1, atom, LIT(1.0));
        const REAL m0 = tissue(c->m0, atom, LIT(1.0));
        const REAL eff = tissue(c->inversion, atom, LIT(1.0));
        for (int64_t e = 0; e < c->event_count; ++e) {
            const REAL dt = (REAL)duration[e];
            const REAL e1 = EXP(-r1 * dt);
            const REAL e2 = EXP(-r2 * dt);
            for (int64_t s = 0; s < S; ++s) {
                plus[s] *= e2;
                minus[s] *= e2;
                lon[s] *= e1;
            }
            lon[0] += LIT(1.0) - e1;
            const uint8_t a = c->action[e];
            if (a & A_PRE_SHIFT) shift(plus, minus, S);
            if (c->kind[e] == 1) {
                if (a & A_INVERSION) {
                    const REAL f = -eff;
                    for (int64_t s = 0; s < S; ++s) lon[s] *= f;
                } else {
                    const REAL alpha = (REAL)flip[e] * b1;
                    const REAL co = COS(alpha);
                    const REAL si = SIN(alpha);
                    const REAL ch = LIT(0.5) * (LIT(1.0) + co);
                    const REAL sh = LIT(0.5) * (LIT(1.0) - co);
                    const REAL hs = LIT(0.5) * si;
                    for (int64_t s = 0; s < S; ++s) {
                        const REAL p = plus[s], m = minus[s], z = lon[s];
                        plus[s] = ch * p + sh * m - si * z;
                        minus[s] = sh * p + ch * m + si * z;
                        lon[s] = hs * p - hs * m + co * z;
                    }
                }
            } else if (c->kind[e] == 2 && (a & A_RECORD)) {
                const int64_t idx = out_base + c->output_index[e];
                out_real[idx] = LIT(0.0);
                out_imag[idx] = m0 * plus[0];
            }
            if (a & A_POST_SHIFT) shift(plus, minus, S);
            if (a & A_SPOIL_AFTER) {
                for (int64_t s = 0; s < S; ++s) plus[s] = minus[s] = LIT(0.0);
            } else if (a & A_SHIFT_AFTER) {
                shift(plus, minus, S);
            }
        }
    }
    free(plus);
}

/* One forward-mode tangent, written as the tangent of the recorded sample
 * only (_epg_cpu.cpp:3136-3285). */
static void run_tangent(const oracle_case* c, const oracle_direction* d,
                        int64_t begin, int64_t end, REAL* out_real, REAL* out_imag) {
    const int64_t S = c->state_count;
    REAL* buf = (REAL*)calloc((size_t)(6 * S), sizeof(REAL));
    REAL *plus = buf, *minus = buf + S, *lon = buf + 2 * S;
    REAL *dp_ = buf + 3 * S, *dm_ = buf + 4 * S, *dz_ = buf + 5 * S;
    for (int64_t work = begin; work < end; ++work) {
        const int64_t train = work / c->atom_count;
        const int64_t atom = work % c->atom_count;
        const int64_t ebase = train * c->event_count;
        const float* duration = c->duration_s + ebase;
        const float* flip = c->flip_rad + ebase;
        const int64_t out_base = (train * c->atom_count + atom) * c->output_count;
        memset(buf, 0, sizeof(REAL) * (size_t)(6 * S));
        lon[0] = LIT(1.0);
        const REAL t1 = (REAL)c->t1_ms[atom];
        const REAL t2 = (REAL)c->t2_ms[atom];
        const REAL r1 = LIT(1000.0) / t1;
        const REAL r2 = LIT(1000.0) / t2;
        const REAL b1 = tissue(c->b1, atom, LIT(1.0));
        const REAL m0 = tissue(c->m0, atom, LIT(1.0));
        const REAL eff = tissue(c->inversion, atom, LIT(1.0));
        const REAL dt1 = tissue(d->t1_ms, atom, LIT(0.0));
        const REAL dt2 = tissue(d->t2_ms, atom, LIT(0.0));
        const REAL db1 = c->b1 ? tissue(d->b1, atom, LIT(0.0)) : LIT(0.0);
        const REAL dm0 = tissue(d->m0, atom, LIT(0.0));
        const REAL deff = c->inversion ? tissue(d->inversion, atom, LIT(0.0)) : LIT(0.0);
        for (int64_t e = 0; e < c->event_count; ++e) {
            const REAL dt = (REAL)duration[e];
            const REAL ddt = d->duration_s ? (REAL)d->duration_s[ebase + e] : LIT(0.0);
            const REAL e1 = EXP(-r1 * dt);
            const REAL e2 = EXP(-r2 * dt);
            const REAL e1t = e1 * (LIT(1000.0) * dt * dt1 / (t1 * t1) - r1 * ddt);
            const REAL e2t = e2 * (LIT(1000.0) * dt * dt2 / (t2 * t2) - r2 * ddt);
            for (int64_t s = 0; s < S; ++s) {
                dp_[s] = dp_[s] * e2 + plus[s] * e2t;
                plus[s] *= e2;
                dm_[s] = dm_[s] * e2 + minus[s] * e2t;
                minus[s] *= e2;
                dz_[s] = dz_[s] * e1 + lon[s] * e1t;
                lon[s] *= e1;
            }
            lon[0] += LIT(1.0) - e1;
            dz_[0] -= e1t;
            const uint8_t a = c->action[e];
            if (a & A_PRE_SHIFT) {
                shift(plus, minus, S);
                shift(dp_, dm_, S);
            }
            if (c->kind[e] == 1) {
                if (a & A_INVERSION) {
                    const REAL f = -eff;
                    const REAL ft = -deff;
                    for (int64_t s = 0; s < S; ++s) {
                        dz_[s] = dz_[s] * f + lon[s] * ft;
                        lon[s] *= f;
                    }
                } else {
                    const REAL fl = (REAL)flip[e];
                    const REAL dfl = d->flip_rad ? (REAL)d->flip_rad[ebase + e] : LIT(0.0);
                    const REAL alpha = fl * b1;
                    const REAL at = dfl * b1 + fl * db1;
                    const REAL co = COS(alpha), si = SIN(alpha);
                    const REAL ch = LIT(0.5) * (LIT(1.0) + co);
                    const REAL sh = LIT(0.5) * (LIT(1.0) - co);
                    const REAL hs = LIT(0.5) * si;
                    const REAL cot = -si * at, sit = co * at;
                    const REAL cht = LIT(-0.5) * si * at;
                    const REAL sht = LIT(0.5) * si * at;
                    const REAL hst = LIT(0.5) * co * at;
                    for (int64_t s = 0; s < S; ++s) {
                        const REAL p = plus[s], m = minus[s], z = lon[s];
                        const REAL dp = dp_[s], dm = dm_[s], dz = dz_[s];
                        dp_[s] = ch * dp + cht * p + sh * dm + sht * m - si * dz - sit * z;
                        dm_[s] = sh * dp + sht * p + ch * dm + cht * m + si * dz + sit * z;
                        dz_[s] = hs * dp + hst * p - hs * dm - hst * m + co * dz + cot * z;
                        plus[s] = ch * p + sh * m - si * z;
                        minus[s] = sh * p + ch * m + si * z;
                        lon[s] = hs * p - hs * m + co * z;
                    }
                }
            } else if (c->kind[e] == 2 && (a & A_RECORD)) {
                const int64_t idx = out_base + c->output_index[e];
                out_real[idx] = LIT(0.0);
                out_imag[idx] = dm0 * plus[0] + m0 * dp_[0];
            }
            if (a & A_POST_SHIFT) {
                shift(plus, minus, S);
                shift(dp_, dm_, S);
            }
            if (a & A_SPOIL_AFTER) {
                for (int64_t s = 0; s < S; ++s) plus[s] = minus[s] = dp_[s] = dm_[s] = LIT(0.0);
            } else if (a & A_SHIFT_AFTER) {
                shift(plus, minus, S);
                shift(dp_, dm_, S);
            }
        }
    }
    free(buf);
}

/* The same tangent with eight atoms of one train side by side
 * (_epg_cpu.cpp:3286-3500 lane helpers, 3503-3695 the kernel): the layout the
 * reference's CPU kernel picks for any run with eight atoms or more on the
 * real subspace (_epg_cpu.cpp:10957-10965), so that the timed CPU baseline runs
 * at the reference's speed. Orders are stored [order][lane]; every per-atom
 * quantity is a lane vector, every event value a splat. The lane vector is
 * GCC's generic vector extension, lowered to whatever SIMD the host has (two
 * 128-bit NEON registers on aarch64, one AVX register on x86). A partial block
 * repeats its first atom into the idle lanes, which are not written back.
 * The derivative factors are formed in the kernel's own order
 * (t1_scale = 1000*dT1/T1^2, then e1' = e1*(dt*t1_scale - r1*ddt)), so the FP32
 * variant matches the reference's lane kernel, which rounds differently from
 * the per-atom one above. Work items are (train, block of eight atoms),
 * train-major. */
#define OLANES 8
typedef REAL lanes_t __attribute__((vector_size(sizeof(REAL) * OLANES)));
/* The same vector at the alignment of one element: the state planes are
 * addressed eight elements at a time from a plain array. */
typedef REAL lanes_at __attribute__((vector_size(sizeof(REAL) * OLANES), aligned(sizeof(REAL))));

static inline lanes_t lanes_ld(const REAL* p) { return *(const lanes_at*)p; }
static inline void lanes_st(REAL* p, lanes_t v) { *(lanes_at*)p = v; }
static inline lanes_t lanes_all(REAL x) {
    lanes_t v;
    for (int l = 0; l < OLANES; ++l) v[l] = x;
    return v;
}

static void shift_lanes(REAL* plus, REAL* minus, int64_t states) {
    for (int64_t s = 0; s + 1 < states; ++s) lanes_st(minus + s * OLANES, lanes_ld(minus + (s + 1) * OLANES));
    lanes_st(minus + (states - 1) * OLANES, lanes_all(LIT(0.0)));
    for (int64_t s = states - 1; s > 0; --s) lanes_st(plus + s * OLANES, lanes_ld(plus + (s - 1) * OLANES));
    lanes_st(plus, -lanes_ld(minus));
}

/* One property for the eight lanes of the block starting at `first`; a null
 * pointer (or an undeclared feature) reads as `identity`. */
static lanes_t gather8(const float* p, int present, REAL identity, int64_t first, int64_t active) {
    lanes_t v;
    for (int l = 0; l < OLANES; ++l) v[l] = (present && p) ? (REAL)p[first + (l < active ? l : 0)] : identity;
    return v;
}

static void run_tangent_lanes(const oracle_case* c, const oracle_direction* d,
                              int64_t begin, int64_t end, REAL* out_real, REAL* out_imag) {
    const int64_t S = c->state_count;
    const int64_t W = S * OLANES;
    const int64_t blocks = (c->atom_count + OLANES - 1) / OLANES;
    REAL* buf = (REAL*)aligned_alloc(64, sizeof(REAL) * (size_t)(6 * W));
    REAL *plus = buf, *minus = buf + W, *lon = buf + 2 * W;
    REAL *dplus = buf + 3 * W, *dminus = buf + 4 * W, *dlon = buf + 5 * W;
    const lanes_t half = lanes_all(LIT(0.5)), one = lanes_all(LIT(1.0));
    for (int64_t work = begin; work < end; ++work) {
        const int64_t train = work / blocks;
        const int64_t first = (work % blocks) * OLANES;
        const int64_t active = c->atom_count - first < OLANES ? c->atom_count - first : OLANES;
        const int64_t ebase = train * c->event_count;
        memset(buf, 0, sizeof(REAL) * (size_t)(6 * W));
        lanes_st(lon, one);
        const lanes_t t1 = gather8(c->t1_ms, 1, LIT(1.0), first, active);
        const lanes_t t2 = gather8(c->t2_ms, 1, LIT(1.0), first, active);
        const lanes_t dt1 = gather8(d->t1_ms, 1, LIT(0.0), first, active);
        const lanes_t dt2 = gather8(d->t2_ms, 1, LIT(0.0), first, active);
        const lanes_t b1 = gather8(c->b1, 1, LIT(1.0), first, active);
        const lanes_t db1 = gather8(d->b1, c->b1 != NULL, LIT(0.0), first, active);
        const lanes_t m0 = gather8(c->m0, 1, LIT(1.0), first, active);
        const lanes_t dm0 = gather8(d->m0, 1, LIT(0.0), first, active);
        const lanes_t flipz = -gather8(c->inversion, 1, LIT(1.0), first, active);
        const lanes_t dflipz = -gather8(d->inversion, c->inversion != NULL, LIT(0.0), first, active);
        const lanes_t r1 = lanes_all(LIT(1000.0)) / t1;
        const lanes_t r2 = lanes_all(LIT(1000.0)) / t2;
        const lanes_t s1 = lanes_all(LIT(1000.0)) * dt1 / (t1 * t1);
        const lanes_t s2 = lanes_all(LIT(1000.0)) * dt2 / (t2 * t2);
        for (int64_t e = 0; e < c->event_count; ++e) {
            const REAL dt = (REAL)c->duration_s[ebase + e];
            const REAL ddt = d->duration_s ? (REAL)d->duration_s[ebase + e] : LIT(0.0);
            lanes_t e1, e2;
            for (int l = 0; l < OLANES; ++l) {
                e1[l] = EXP(-r1[l] * dt);
                e2[l] = EXP(-r2[l] * dt);
            }
            const lanes_t e1t = e1 * (dt * s1 - r1 * ddt);
            const lanes_t e2t = e2 * (dt * s2 - r2 * ddt);
            for (int64_t s = 0; s < S; ++s) {
                REAL* o = buf + s * OLANES;
                const lanes_t p = lanes_ld(o), m = lanes_ld(o + W), z = lanes_ld(o + 2 * W);
                lanes_st(o + 3 * W, lanes_ld(o + 3 * W) * e2 + p * e2t);
                lanes_st(o, p * e2);
                lanes_st(o + 4 * W, lanes_ld(o + 4 * W) * e2 + m * e2t);
                lanes_st(o + W, m * e2);
                lanes_st(o + 5 * W, lanes_ld(o + 5 * W) * e1 + z * e1t);
                lanes_st(o + 2 * W, z * e1);
            }
            lanes_st(lon, lanes_ld(lon) + (one - e1));
            lanes_st(dlon, lanes_ld(dlon) - e1t);
            const uint8_t a = c->action[e];
            if (a & A_PRE_SHIFT) {
                shift_lanes(plus, minus, S);
                shift_lanes(dplus, dminus, S);
            }
            if (c->kind[e] == 1) {
                if (a & A_INVERSION) {
                    for (int64_t s = 0; s < S; ++s) {
                        REAL* o = buf + s * OLANES;
                        const lanes_t z = lanes_ld(o + 2 * W);
                        lanes_st(o + 5 * W, lanes_ld(o + 5 * W) * flipz + z * dflipz);
                        lanes_st(o + 2 * W, z * flipz);
                    }
                } else {
                    const REAL fl = (REAL)c->flip_rad[ebase + e];
                    const REAL dfl = d->flip_rad ? (REAL)d->flip_rad[ebase + e] : LIT(0.0);
                    lanes_t co, si, at;
                    for (int l = 0; l < OLANES; ++l) {
                        const REAL alpha = fl * b1[l];
                        co[l] = COS(alpha);
                        si[l] = SIN(alpha);
                        at[l] = dfl * b1[l] + fl * db1[l];
                    }
                    const lanes_t ch = half * (one + co), sh = half * (one - co), hs = half * si;
                    const lanes_t cot = -(si * at), sit = co * at;
                    const lanes_t cht = half * cot, sht = -(half * cot), hst = half * sit;
                    for (int64_t s = 0; s < S; ++s) {
                        REAL* o = buf + s * OLANES;
                        const lanes_t p = lanes_ld(o), m = lanes_ld(o + W), z = lanes_ld(o + 2 * W);
                        const lanes_t dp = lanes_ld(o + 3 * W), dm = lanes_ld(o + 4 * W),
                                      dz = lanes_ld(o + 5 * W);
                        lanes_st(o + 3 * W, ch * dp + cht * p + sh * dm + sht * m - si * dz - sit * z);
                        lanes_st(o + 4 * W, sh * dp + sht * p + ch * dm + cht * m + si * dz + sit * z);
                        lanes_st(o + 5 * W, hs * dp + hst * p - hs * dm - hst * m + co * dz + cot * z);
                        lanes_st(o, ch * p + sh * m - si * z);
                        lanes_st(o + W, sh * p + ch * m + si * z);
                        lanes_st(o + 2 * W, hs * p - hs * m + co * z);
                    }
                }
            } else if (c->kind[e] == 2 && (a & A_RECORD)) {
                for (int64_t l = 0; l < active; ++l) {
                    const int64_t idx = (train * c->atom_count + first + l) * c->output_count
                                        + c->output_index[e];
                    out_real[idx] = LIT(0.0);
                    out_imag[idx] = dm0[l] * plus[l] + m0[l] * dplus[l];
                }
            }
            if (a & A_POST_SHIFT) {
                shift_lanes(plus, minus, S);
                shift_lanes(dplus, dminus, S);
            }
            if (a & A_SPOIL_AFTER) {
                memset(plus, 0, sizeof(REAL) * (size_t)(2 * W));
                memset(dplus, 0, sizeof(REAL) * (size_t)(2 * W));
            } else if (a & A_SHIFT_AFTER) {
                shift_lanes(plus, minus, S);
                shift_lanes(dplus, dminus, S);
            }
        }
    }
    free(buf);
}

/* First-order adjoint (_epg_cpu.cpp:5985-6232): the entry state of every
 * event is recorded, then the events are swept backwards. Gradients add into
 * the given arrays: per atom for t1, t2, m0, b1, inversion; per (train,
 * event) for flip and duration. Only the imaginary seed plane acts. */
static void run_adjoint(const oracle_case* c, const float* seed_imag,
                        int64_t begin, int64_t end,
                        REAL* g_t1, REAL* g_t2, REAL* g_m0, REAL* g_b1, REAL* g_inv,
                        REAL* g_flip, REAL* g_duration) {
    const int64_t S = c->state_count;
    const int64_t E = c->event_count;
    REAL* traj = (REAL*)malloc(sizeof(REAL) * (size_t)(E > 0 ? E : 1) * (size_t)(3 * S));
    REAL* buf = (REAL*)calloc((size_t)(9 * S), sizeof(REAL));
    REAL *plus = buf, *minus = buf + S, *lon = buf + 2 * S;
    REAL *pb = buf + 3 * S, *mb = buf + 4 * S, *zb = buf + 5 * S;
    REAL *ps = buf + 6 * S, *ms = buf + 7 * S, *zs = buf + 8 * S;
    for (int64_t work = begin; work < end; ++work) {
        const int64_t train = work / c->atom_count;
        const int64_t atom = work % c->atom_count;
        const int64_t ebase = train * E;
        const float* duration = c->duration_s + ebase;
        const float* flip = c->flip_rad + ebase;
        const int64_t out_base = (train * c->atom_count + atom) * c->output_count;
        const REAL t1 = (REAL)c->t1_ms[atom];
        const REAL t2 = (REAL)c->t2_ms[atom];
        const REAL m0 = tissue(c->m0, atom, LIT(1.0));
        const REAL b1 = tissue(c->b1, atom, LIT(1.0));
        const REAL eff = tissue(c->inversion, atom, LIT(1.0));
        const REAL r1 = LIT(1000.0) / t1;
        const REAL r2 = LIT(1000.0) / t2;
        memset(buf, 0, sizeof(REAL) * (size_t)(9 * S));
        lon[0] = LIT(1.0);
        for (int64_t e = 0; e < E; ++e) {
            REAL* slot = traj + e * 3 * S;
            memcpy(slot, plus, sizeof(REAL) * (size_t)(3 * S));
            const REAL dt = (REAL)duration[e];
            const REAL e1 = EXP(-r1 * dt), e2 = EXP(-r2 * dt);
            for (int64_t s = 0; s < S; ++s) {
                plus[s] *= e2;
                minus[s] *= e2;
                lon[s] *= e1;
            }
            lon[0] += LIT(1.0) - e1;
            const uint8_t a = c->action[e];
            if (a & A_PRE_SHIFT) shift(plus, minus, S);
            if (c->kind[e] == 1) {
                if (a & A_INVERSION) {
                    for (int64_t s = 0; s < S; ++s) lon[s] *= -eff;
                } else {
                    const REAL alpha = (REAL)flip[e] * b1;
                    const REAL co = COS(alpha), si = SIN(alpha);
                    const REAL ch = LIT(0.5) * (LIT(1.0) + co);
                    const REAL sh = LIT(0.5) * (LIT(1.0) - co);
                    const REAL hs = LIT(0.5) * si;
                    for (int64_t s = 0; s < S; ++s) {
                        const REAL p = plus[s], m = minus[s], z = lon[s];
                        plus[s] = ch * p + sh * m - si * z;
                        minus[s] = sh * p + ch * m + si * z;
                        lon[s] = hs * p - hs * m + co * z;
                    }
                }
            }
            if (a & A_POST_SHIFT) shift(plus, minus, S);
            if (a & A_SPOIL_AFTER) {
                for (int64_t s = 0; s < S; ++s) plus[s] = minus[s] = LIT(0.0);
            } else if (a & A_SHIFT_AFTER) {
                shift(plus, minus, S);
            }
        }
        for (int64_t s = 0; s < 3 * S; ++s) pb[s] = LIT(0.0);
        REAL gt1 = 0, gt2 = 0, gm0 = 0, gb1 = 0, ginv = 0;
        for (int64_t e = E - 1; e >= 0; --e) {
            const REAL* slot = traj + e * 3 * S;
            const uint8_t a = c->action[e];
            const REAL dt = (REAL)duration[e];
            const REAL e1 = EXP(-r1 * dt), e2 = EXP(-r2 * dt);
            for (int64_t s = 0; s < S; ++s) {
                ps[s] = slot[s] * e2;
                ms[s] = slot[S + s] * e2;
                zs[s] = slot[2 * S + s] * e1;
            }
            zs[0] += LIT(1.0) - e1;
            if (a & A_PRE_SHIFT) shift(ps, ms, S);
            if (a & A_SPOIL_AFTER) {
                for (int64_t s = 0; s < S; ++s) pb[s] = mb[s] = LIT(0.0);
            } else if (a & A_SHIFT_AFTER) {
                shift_adjoint(pb, mb, S);
            }
            if (a & A_POST_SHIFT) shift_adjoint(pb, mb, S);
            if (c->kind[e] == 1) {
                if (a & A_INVERSION) {
                    for (int64_t s = 0; s < S; ++s) {
                        ginv -= zb[s] * zs[s];
                        zb[s] *= -eff;
                    }
                } else {
                    const REAL fl = (REAL)flip[e];
                    const REAL alpha = fl * b1;
                    const REAL co = COS(alpha), si = SIN(alpha);
                    const REAL ch = LIT(0.5) * (LIT(1.0) + co);
                    const REAL sh = LIT(0.5) * (LIT(1.0) - co);
                    const REAL hs = LIT(0.5) * si;
                    REAL ga = LIT(0.0);
                    for (int64_t s = 0; s < S; ++s) {
                        const REAL p = ps[s], m = ms[s], z = zs[s];
                        const REAL pbs = pb[s], mbs = mb[s], zbs = zb[s];
                        ga += pbs * (hs * m - hs * p - co * z)
                            + mbs * (hs * p - hs * m + co * z)
                            + zbs * (LIT(0.5) * co * p - LIT(0.5) * co * m - si * z);
                        pb[s] = ch * pbs + sh * mbs + hs * zbs;
                        mb[s] = sh * pbs + ch * mbs - hs * zbs;
                        zb[s] = -si * pbs + si * mbs + co * zbs;
                    }
                    g_flip[ebase + e] += ga * b1;
                    gb1 += ga * fl;
                }
            } else if (c->kind[e] == 2 && (a & A_RECORD)) {
                const REAL sd = (REAL)seed_imag[out_base + c->output_index[e]];
                gm0 += sd * ps[0];
                pb[0] += sd * m0;
            }
            if (a & A_PRE_SHIFT) shift_adjoint(pb, mb, S);
            REAL ge1 = -zb[0];
            REAL ge2 = LIT(0.0);
            for (int64_t s = 0; s < S; ++s) {
                ge2 += pb[s] * slot[s] + mb[s] * slot[S + s];
                ge1 += zb[s] * slot[2 * S + s];
                pb[s] *= e2;
                mb[s] *= e2;
                zb[s] *= e1;
            }
            gt1 += ge1 * (e1 * dt * (LIT(1000.0) / (t1 * t1)));
            gt2 += ge2 * (e2 * dt * (LIT(1000.0) / (t2 * t2)));
            g_duration[ebase + e] += -ge1 * (r1 * e1) - ge2 * (r2 * e2);
        }
        g_t1[atom] += gt1;
        g_t2[atom] += gt2;
        g_m0[atom] += gm0;
        g_b1[atom] += gb1;
        g_inv[atom] += ginv;
    }
    free(buf);
    free(traj);
}

/* ---- second order: forward over reverse ---------------------------------- */

/* A value and its derivative along one direction, with the reference's
 * DualFloat products (_epg_cpu.cpp:346-365): the tangent of a*b is
 * a.t*b.v + a.v*b.t, in that order. */
typedef struct {
    REAL v, t;
} dual;

static inline dual dl(REAL v, REAL t) {
    dual r;
    r.v = v;
    r.t = t;
    return r;
}
static inline dual dadd(dual a, dual b) { return dl(a.v + b.v, a.t + b.t); }
static inline dual dsub(dual a, dual b) { return dl(a.v - b.v, a.t - b.t); }
static inline dual dmul(dual a, dual b) { return dl(a.v * b.v, a.t * b.v + a.v * b.t); }
static inline dual dscale(REAL a, dual b) { return dl(a * b.v, a * b.t); }
static inline dual dexp(dual a) {
    const REAL v = EXP(a.v);
    return dl(v, v * a.t);
}
static inline dual dinv_square(dual a) {
    const REAL inverse = LIT(1.0) / (a.v * a.v);
    return dl(inverse, LIT(-2.0) * a.t * inverse / a.v);
}

static void dshift(dual* plus, dual* minus, int64_t states) {
    for (int64_t s = 0; s + 1 < states; ++s) minus[s] = minus[s + 1];
    minus[states - 1] = dl(LIT(0.0), LIT(0.0));
    for (int64_t s = states - 1; s > 0; --s) plus[s] = plus[s - 1];
    plus[0] = dsub(dl(LIT(0.0), LIT(0.0)), minus[0]);
}

static void dshift_adjoint(dual* plus_bar, dual* minus_bar, int64_t states) {
    const dual carry = dsub(dl(LIT(0.0), LIT(0.0)), plus_bar[0]);
    for (int64_t s = 0; s + 1 < states; ++s) plus_bar[s] = plus_bar[s + 1];
    plus_bar[states - 1] = dl(LIT(0.0), LIT(0.0));
    for (int64_t s = states - 1; s > 0; --s) minus_bar[s] = minus_bar[s - 1];
    minus_bar[0] = dl(LIT(0.0), LIT(0.0));
    if (states > 1) minus_bar[1] = dadd(minus_bar[1], carry);
}

/* The first-order adjoint run in dual numbers along direction d, with the
 * seed on the imaginary output plane (_epg_cpu.cpp:7028-7330): the value
 * parts of the gradients are J^T seed (the gradient with respect to the
 * direction), the tangent parts the derivative of that along d (the
 * curvature, the gradient of <seed, J d> with respect to the inputs).
 * Gradients add into value[7] and curve[7], each ordered t1, t2, m0, b1,
 * inversion (per atom), flip, duration (per train and event). Tissue
 * directions follow the reference's feature flags: m0, b1 and inversion
 * carry their direction only where the property itself is given. */
static void run_second(const oracle_case* c, const oracle_direction* d, const float* seed_imag,
                       int64_t begin, int64_t end, REAL* const* value, REAL* const* curve) {
    const int64_t S = c->state_count;
    const int64_t E = c->event_count;
    const dual zero = dl(LIT(0.0), LIT(0.0));
    const dual one = dl(LIT(1.0), LIT(0.0));
    dual* traj = (dual*)malloc(sizeof(dual) * (size_t)(E > 0 ? E : 1) * (size_t)(3 * S));
    dual* buf = (dual*)calloc((size_t)(9 * S), sizeof(dual));
    dual *plus = buf, *minus = buf + S, *lon = buf + 2 * S;
    dual *pb = buf + 3 * S, *mb = buf + 4 * S, *zb = buf + 5 * S;
    dual *ps = buf + 6 * S, *ms = buf + 7 * S, *zs = buf + 8 * S;
    for (int64_t work = begin; work < end; ++work) {
        const int64_t train = work / c->atom_count;
        const int64_t atom = work % c->atom_count;
        const int64_t ebase = train * E;
        const float* duration = c->duration_s + ebase;
        const float* flip = c->flip_rad + ebase;
        const int64_t out_base = (train * c->atom_count + atom) * c->output_count;
        const dual t1 = dl((REAL)c->t1_ms[atom], tissue(d->t1_ms, atom, LIT(0.0)));
        const dual t2 = dl((REAL)c->t2_ms[atom], tissue(d->t2_ms, atom, LIT(0.0)));
        const dual m0 = c->m0 ? dl((REAL)c->m0[atom], tissue(d->m0, atom, LIT(0.0))) : one;
        const dual b1 = c->b1 ? dl((REAL)c->b1[atom], tissue(d->b1, atom, LIT(0.0))) : one;
        const dual inversion =
            c->inversion ? dl((REAL)c->inversion[atom], tissue(d->inversion, atom, LIT(0.0)))
                         : one;
        const dual r1 = dl(LIT(1000.0) / t1.v, LIT(-1000.0) * t1.t / (t1.v * t1.v));
        const dual r2 = dl(LIT(1000.0) / t2.v, LIT(-1000.0) * t2.t / (t2.v * t2.v));
        for (int64_t s = 0; s < 9 * S; ++s) buf[s] = zero;
        lon[0] = one;
        for (int64_t e = 0; e < E; ++e) {
            dual* slot = traj + e * 3 * S;
            memcpy(slot, plus, sizeof(dual) * (size_t)(3 * S));
            const dual dt = dl((REAL)duration[e],
                               d->duration_s ? (REAL)d->duration_s[ebase + e] : LIT(0.0));
            const dual e1 = dexp(dsub(zero, dmul(r1, dt)));
            const dual e2 = dexp(dsub(zero, dmul(r2, dt)));
            for (int64_t s = 0; s < S; ++s) {
                plus[s] = dmul(plus[s], e2);
                minus[s] = dmul(minus[s], e2);
                lon[s] = dmul(lon[s], e1);
            }
            lon[0] = dadd(lon[0], dsub(one, e1));
            const uint8_t a = c->action[e];
            if (a & A_PRE_SHIFT) dshift(plus, minus, S);
            if (c->kind[e] == 1) {
                if (a & A_INVERSION) {
                    const dual efficiency = dsub(zero, inversion);
                    for (int64_t s = 0; s < S; ++s) lon[s] = dmul(lon[s], efficiency);
                } else {
                    const dual fl = dl((REAL)flip[e],
                                       d->flip_rad ? (REAL)d->flip_rad[ebase + e] : LIT(0.0));
                    const dual alpha = dmul(fl, b1);
                    const dual co = dl(COS(alpha.v), -SIN(alpha.v) * alpha.t);
                    const dual si = dl(SIN(alpha.v), COS(alpha.v) * alpha.t);
                    const dual ch = dscale(LIT(0.5), dadd(one, co));
                    const dual sh = dscale(LIT(0.5), dsub(one, co));
                    const dual hs = dscale(LIT(0.5), si);
                    for (int64_t s = 0; s < S; ++s) {
                        const dual p = plus[s], m = minus[s], z = lon[s];
                        plus[s] = dsub(dadd(dmul(ch, p), dmul(sh, m)), dmul(si, z));
                        minus[s] = dadd(dadd(dmul(sh, p), dmul(ch, m)), dmul(si, z));
                        lon[s] = dadd(dsub(dmul(hs, p), dmul(hs, m)), dmul(co, z));
                    }
                }
            }
            if (a & A_POST_SHIFT) dshift(plus, minus, S);
            if (a & A_SPOIL_AFTER) {
                for (int64_t s = 0; s < S; ++s) plus[s] = minus[s] = zero;
            } else if (a & A_SHIFT_AFTER) {
                dshift(plus, minus, S);
            }
        }
        for (int64_t s = 0; s < 3 * S; ++s) pb[s] = zero;
        dual gt1 = zero, gt2 = zero, gm0 = zero, gb1 = zero, ginv = zero;
        for (int64_t e = E - 1; e >= 0; --e) {
            const dual* slot = traj + e * 3 * S;
            const uint8_t a = c->action[e];
            const dual dt = dl((REAL)duration[e],
                               d->duration_s ? (REAL)d->duration_s[ebase + e] : LIT(0.0));
            const dual e1 = dexp(dsub(zero, dmul(r1, dt)));
            const dual e2 = dexp(dsub(zero, dmul(r2, dt)));
            for (int64_t s = 0; s < S; ++s) {
                ps[s] = dmul(slot[s], e2);
                ms[s] = dmul(slot[S + s], e2);
                zs[s] = dmul(slot[2 * S + s], e1);
            }
            zs[0] = dadd(zs[0], dsub(one, e1));
            if (a & A_PRE_SHIFT) dshift(ps, ms, S);
            if (a & A_SPOIL_AFTER) {
                for (int64_t s = 0; s < S; ++s) pb[s] = mb[s] = zero;
            } else if (a & A_SHIFT_AFTER) {
                dshift_adjoint(pb, mb, S);
            }
            if (a & A_POST_SHIFT) dshift_adjoint(pb, mb, S);
            if (c->kind[e] == 1) {
                if (a & A_INVERSION) {
                    const dual efficiency = dsub(zero, inversion);
                    for (int64_t s = 0; s < S; ++s) {
                        ginv = dsub(ginv, dmul(zb[s], zs[s]));
                        zb[s] = dmul(zb[s], efficiency);
                    }
                } else {
                    const dual fl = dl((REAL)flip[e],
                                       d->flip_rad ? (REAL)d->flip_rad[ebase + e] : LIT(0.0));
                    const dual alpha = dmul(fl, b1);
                    const dual co = dl(COS(alpha.v), -SIN(alpha.v) * alpha.t);
                    const dual si = dl(SIN(alpha.v), COS(alpha.v) * alpha.t);
                    const dual ch = dscale(LIT(0.5), dadd(one, co));
                    const dual sh = dscale(LIT(0.5), dsub(one, co));
                    const dual hs = dscale(LIT(0.5), si);
                    const dual hco = dscale(LIT(0.5), co);
                    dual ga = zero;
                    for (int64_t s = 0; s < S; ++s) {
                        const dual p = ps[s], m = ms[s], z = zs[s];
                        const dual pbs = pb[s], mbs = mb[s], zbs = zb[s];
                        ga = dadd(dadd(dadd(ga, dmul(pbs, dsub(dsub(dmul(hs, m), dmul(hs, p)),
                                                                dmul(co, z)))),
                                       dmul(mbs, dadd(dsub(dmul(hs, p), dmul(hs, m)), dmul(co, z)))),
                                  dmul(zbs, dsub(dsub(dmul(hco, p), dmul(hco, m)), dmul(si, z))));
                        pb[s] = dadd(dadd(dmul(ch, pbs), dmul(sh, mbs)), dmul(hs, zbs));
                        mb[s] = dsub(dadd(dmul(sh, pbs), dmul(ch, mbs)), dmul(hs, zbs));
                        zb[s] = dadd(dadd(dmul(dsub(zero, si), pbs), dmul(si, mbs)), dmul(co, zbs));
                    }
                    const dual gf = dmul(ga, b1);
                    value[5][ebase + e] += gf.v;
                    curve[5][ebase + e] += gf.t;
                    gb1 = dadd(gb1, dmul(ga, fl));
                }
            } else if (c->kind[e] == 2 && (a & A_RECORD)) {
                const dual sd = dl((REAL)seed_imag[out_base + c->output_index[e]], LIT(0.0));
                gm0 = dadd(gm0, dmul(sd, ps[0]));
                pb[0] = dadd(pb[0], dmul(sd, m0));
            }
            if (a & A_PRE_SHIFT) dshift_adjoint(pb, mb, S);
            dual ge1 = dsub(zero, zb[0]);
            dual ge2 = zero;
            for (int64_t s = 0; s < S; ++s) {
                ge2 = dadd(dadd(ge2, dmul(pb[s], slot[s])), dmul(mb[s], slot[S + s]));
                ge1 = dadd(ge1, dmul(zb[s], slot[2 * S + s]));
                pb[s] = dmul(pb[s], e2);
                mb[s] = dmul(mb[s], e2);
                zb[s] = dmul(zb[s], e1);
            }
            const dual scale1 = dmul(dmul(e1, dt), dscale(LIT(1000.0), dinv_square(t1)));
            const dual scale2 = dmul(dmul(e2, dt), dscale(LIT(1000.0), dinv_square(t2)));
            gt1 = dadd(gt1, dmul(ge1, scale1));
            gt2 = dadd(gt2, dmul(ge2, scale2));
            /* Atoms of a train add into one slot per event, in this order. */
            const dual acc = dl(value[6][ebase + e], curve[6][ebase + e]);
            const dual gd = dsub(dsub(acc, dmul(ge1, dmul(r1, e1))), dmul(ge2, dmul(r2, e2)));
            value[6][ebase + e] = gd.v;
            curve[6][ebase + e] = gd.t;
        }
        const dual g[5] = {gt1, gt2, gm0, gb1, ginv};
        for (int k = 0; k < 5; ++k) {
            value[k][atom] += g[k].v;
            curve[k][atom] += g[k].t;
        }
    }
    free(buf);
    free(traj);
}

/* ---- the complex path (one pool, instant RF) ---------------------------- */

/* Per-event RF / receiver phase (train_count*event_count) and the per-voxel
 * transmit phase and off-resonance; each nullable (zero). */
typedef struct {
    const float* phase_rad;
    const float* b1_phase_rad;
    const float* b0_hz;
} oracle_offaxis;

typedef struct {
    REAL re, im;
} cplx;

static inline cplx cmul(cplx a, cplx b) {
    const REAL ac = a.re * b.re, bd = a.im * b.im, ad = a.re * b.im, bc = a.im * b.re;
    cplx r = {ac - bd, ad + bc};
    return r;
}
static inline cplx cadd(cplx a, cplx b) {
    cplx r = {a.re + b.re, a.im + b.im};
    return r;
}
static inline cplx cscale(REAL s, cplx a) {
    cplx r = {s * a.re, s * a.im};
    return r;
}
static inline cplx cconj(cplx a) {
    cplx r = {a.re, -a.im};
    return r;
}
static inline cplx cpolar(REAL rho, REAL theta) {
    cplx r = {rho * COS(theta), rho * SIN(theta)};
    return r;
}

/* F- takes order k+1, F+ takes order k-1, the top F- order is lost and
 * F+[0] is the conjugate of the new F-[0] (_epg_cpu.cpp:2164-2174). */
static void shift_complex(cplx* plus, cplx* minus, int64_t states) {
    for (int64_t s = 0; s + 1 < states; ++s) minus[s] = minus[s + 1];
    const cplx zero = {LIT(0.0), LIT(0.0)};
    minus[states - 1] = zero;
    for (int64_t s = states - 1; s > 0; --s) plus[s] = plus[s - 1];
    plus[0] = cconj(minus[0]);
}

/* The pulse's 3x3 transition with flip alpha and phase phi
 * (_epg_cpu.cpp:2176-2208). */
static void rotate_complex(cplx* plus, cplx* minus, cplx* lon, int64_t states, REAL alpha,
                           REAL phi) {
    const REAL cosine = COS(alpha);
    const REAL sine = SIN(alpha);
    const REAL chs = LIT(0.5) * (LIT(1.0) + cosine);
    const REAL shs = LIT(0.5) * (LIT(1.0) - cosine);
    const cplx one = cpolar(LIT(1.0), phi);
    const cplx two = cmul(one, one);
    const cplx t00 = {chs, LIT(0.0)};
    const cplx t01 = cscale(shs, two);
    const cplx mis = {LIT(0.0), -sine}, pis = {LIT(0.0), sine};
    const cplx mhs = {LIT(0.0), -(LIT(0.5) * sine)}, phs = {LIT(0.0), LIT(0.5) * sine};
    const cplx t02 = cmul(mis, one);
    const cplx t10 = cconj(t01);
    const cplx t11 = t00;
    const cplx t12 = cmul(pis, cconj(one));
    const cplx t20 = cmul(mhs, cconj(one));
    const cplx t21 = cmul(phs, one);
    const cplx t22 = {cosine, LIT(0.0)};
    for (int64_t s = 0; s < states; ++s) {
        const cplx fp = plus[s], fm = minus[s], z = lon[s];
        plus[s] = cadd(cadd(cmul(t00, fp), cmul(t01, fm)), cmul(t02, z));
        minus[s] = cadd(cadd(cmul(t10, fp), cmul(t11, fm)), cmul(t12, z));
        lon[s] = cadd(cadd(cmul(t20, fp), cmul(t21, fm)), cmul(t22, z));
    }
}

/* Transpose of shift_complex: F+ cotangents move one order down, F-
 * cotangents one order up, and F+[0] = conj(F-[0]) returns conj(pb[0]) to
 * the F-[1] that became F-[0]. */
static void shift_complex_adjoint(cplx* pb, cplx* mb, int64_t states) {
    const cplx carry = cconj(pb[0]);
    const cplx zero = {LIT(0.0), LIT(0.0)};
    for (int64_t s = 0; s + 1 < states; ++s) pb[s] = pb[s + 1];
    pb[states - 1] = zero;
    for (int64_t s = states - 1; s > 0; --s) mb[s] = mb[s - 1];
    mb[0] = zero;
    if (states > 1) mb[1] = cadd(mb[1], carry);
}

/* Transpose (conjugate) of rotate_complex applied to the cotangents, and the
 * gradients Re(conj(y_bar) dT/dalpha x), Re(conj(y_bar) dT/dphi x) added
 * into ga, gp, with x the pre-pulse state (p, m, z). */
static void rotate_complex_adjoint(cplx* pb, cplx* mb, cplx* zb, const cplx* p, const cplx* m,
                                   const cplx* z, int64_t states, REAL alpha, REAL phi, REAL* ga,
                                   REAL* gp) {
    const REAL co = COS(alpha), si = SIN(alpha);
    const REAL chs = LIT(0.5) * (LIT(1.0) + co), shs = LIT(0.5) * (LIT(1.0) - co);
    const cplx one = cpolar(LIT(1.0), phi), two = cmul(one, one);
    const cplx i1 = {LIT(0.0), LIT(1.0)};
    /* T and dT/dalpha, dT/dphi, entry by entry. */
    cplx t[3][3], ta[3][3], tp[3][3];
    t[0][0] = (cplx){chs, LIT(0.0)};
    t[0][1] = cscale(shs, two);
    t[0][2] = cmul((cplx){LIT(0.0), -si}, one);
    t[1][0] = cconj(t[0][1]);
    t[1][1] = t[0][0];
    t[1][2] = cmul((cplx){LIT(0.0), si}, cconj(one));
    t[2][0] = cmul((cplx){LIT(0.0), -LIT(0.5) * si}, cconj(one));
    t[2][1] = cmul((cplx){LIT(0.0), LIT(0.5) * si}, one);
    t[2][2] = (cplx){co, LIT(0.0)};
    ta[0][0] = (cplx){-LIT(0.5) * si, LIT(0.0)};
    ta[0][1] = cscale(LIT(0.5) * si, two);
    ta[0][2] = cmul((cplx){LIT(0.0), -co}, one);
    ta[1][0] = cconj(ta[0][1]);
    ta[1][1] = ta[0][0];
    ta[1][2] = cmul((cplx){LIT(0.0), co}, cconj(one));
    ta[2][0] = cmul((cplx){LIT(0.0), -LIT(0.5) * co}, cconj(one));
    ta[2][1] = cmul((cplx){LIT(0.0), LIT(0.5) * co}, one);
    ta[2][2] = (cplx){-si, LIT(0.0)};
    /* d/dphi: one -> i one, two -> 2i two, conj(one) -> -i conj(one). */
    tp[0][0] = (cplx){LIT(0.0), LIT(0.0)};
    tp[0][1] = cmul(cscale(LIT(2.0), i1), t[0][1]);
    tp[0][2] = cmul(i1, t[0][2]);
    tp[1][0] = cmul(cscale(-LIT(2.0), i1), t[1][0]);
    tp[1][1] = tp[0][0];
    tp[1][2] = cmul(cscale(-LIT(1.0), i1), t[1][2]);
    tp[2][0] = cmul(cscale(-LIT(1.0), i1), t[2][0]);
    tp[2][1] = cmul(i1, t[2][1]);
    tp[2][2] = tp[0][0];
    for (int64_t s = 0; s < states; ++s) {
        const cplx x[3] = {p[s], m[s], z[s]};
        const cplx y[3] = {pb[s], mb[s], zb[s]};
        for (int r = 0; r < 3; ++r) {
            cplx da = {LIT(0.0), LIT(0.0)}, dp = {LIT(0.0), LIT(0.0)};
            for (int k = 0; k < 3; ++k) {
                da = cadd(da, cmul(ta[r][k], x[k]));
                dp = cadd(dp, cmul(tp[r][k], x[k]));
            }
            *ga += y[r].re * da.re + y[r].im * da.im;
            *gp += y[r].re * dp.re + y[r].im * dp.im;
        }
        cplx nx[3];
        for (int k = 0; k < 3; ++k) {
            nx[k] = (cplx){LIT(0.0), LIT(0.0)};
            for (int r = 0; r < 3; ++r) nx[k] = cadd(nx[k], cmul(cconj(t[r][k]), y[r]));
        }
        pb[s] = nx[0];
        mb[s] = nx[1];
        zb[s] = nx[2];
    }
}

/* Complex forward over work items [begin, end): both output planes are the
 * recorded m0 * F+[0] demodulated by the receiver phase. */
static void run_forward_complex(const oracle_case* c, const oracle_offaxis* o, int64_t begin,
                                int64_t end, REAL* out_real, REAL* out_imag) {
    const int64_t S = c->state_count;
    cplx* plus = (cplx*)calloc((size_t)(3 * S), sizeof(cplx));
    cplx* minus = plus + S;
    cplx* lon = minus + S;
    const int off_axis = o->b0_hz != NULL || o->b1_phase_rad != NULL;
#if defined(REAL_IS_FLOAT)
    const REAL pi = 3.14159265358979323846F;
#else
    const REAL pi = 3.14159265358979323846;
#endif
    for (int64_t work = begin; work < end; ++work) {
        const int64_t train = work / c->atom_count;
        const int64_t atom = work % c->atom_count;
        const float* duration = c->duration_s + train * c->event_count;
        const float* flip = c->flip_rad + train * c->event_count;
        const float* phase = o->phase_rad ? o->phase_rad + train * c->event_count : NULL;
        const int64_t out_base = (train * c->atom_count + atom) * c->output_count;
        memset(plus, 0, sizeof(cplx) * (size_t)(3 * S));
        lon[0].re = LIT(1.0);
        const REAL r1 = LIT(1000.0) / (REAL)c->t1_ms[atom];
        const REAL r2 = LIT(1000.0) / (REAL)c->t2_ms[atom];
        const REAL b1 = tissue(c->b1, atom, LIT(1.0));
        const REAL m0 = tissue(c->m0, atom, LIT(1.0));
        const REAL eff = tissue(c->inversion, atom, LIT(1.0));
        const REAL b1_phase = tissue(o->b1_phase_rad, atom, LIT(0.0));
        const REAL b0 = tissue(o->b0_hz, atom, LIT(0.0));
        for (int64_t e = 0; e < c->event_count; ++e) {
            const REAL dt = (REAL)duration[e];
            const REAL e1 = EXP(-r1 * dt);
            const REAL e2 = EXP(-r2 * dt);
            const REAL off = off_axis ? -LIT(2.0) * pi * b0 * dt : LIT(0.0);
            cplx transverse = {e2, LIT(0.0)};
            if (off_axis) transverse = cpolar(e2, off);
            const cplx along = {e1, LIT(0.0)};
            for (int64_t s = 0; s < S; ++s) {
                plus[s] = cmul(plus[s], transverse);
                minus[s] = cmul(minus[s], cconj(transverse));
                lon[s] = cmul(lon[s], along);
            }
            lon[0].re += LIT(1.0) - e1;
            const uint8_t a = c->action[e];
            if (a & A_PRE_SHIFT) shift_complex(plus, minus, S);
            if (c->kind[e] == 1) {
                if (a & A_INVERSION) {
                    const REAL f = -eff;
                    for (int64_t s = 0; s < S; ++s) lon[s] = cscale(f, lon[s]);
                } else {
                    const REAL theta = (REAL)flip[e] * b1;
                    const REAL phi = (phase ? (REAL)phase[e] : LIT(0.0)) + b1_phase;
                    rotate_complex(plus, minus, lon, S, theta, phi);
                }
            } else if (c->kind[e] == 2 && (a & A_RECORD)) {
                const int64_t idx = out_base + c->output_index[e];
                const cplx demod = cpolar(LIT(1.0), -(phase ? (REAL)phase[e] : LIT(0.0)));
                const cplx v = cmul(cscale(m0, plus[0]), demod);
                out_real[idx] = v.re;
                out_imag[idx] = v.im;
            }
            if (a & A_POST_SHIFT) shift_complex(plus, minus, S);
            if (a & A_SPOIL_AFTER) {
                const cplx zero = {LIT(0.0), LIT(0.0)};
                for (int64_t s = 0; s < S; ++s) plus[s] = minus[s] = zero;
            } else if (a & A_SHIFT_AFTER) {
                shift_complex(plus, minus, S);
            }
        }
    }
    free(plus);
}

/* First-order adjoint of the complex path (the single-pool instant-RF case
 * of simulate_vjp_range, _epg_cpu.cpp:4840-5985), restated in this file's
 * complex arithmetic: the entry state of every event is recorded, then the
 * events are swept backwards replaying each event's stages from its entry
 * state. The seed is complex (real plane + i imaginary plane): the loss is
 * sum Re(conj(seed) * sample). For y = a x the cotangent is x_bar = conj(a)
 * y_bar; a parameter's gradient is Re(conj(y_bar) * (da/dp) x).
 * Gradients add into g[10]: per atom t1, t2, m0, b1, inversion, b1 phase,
 * b0; per (train, event) flip, duration, phase. */
static void run_adjoint_complex(const oracle_case* c, const oracle_offaxis* o,
                                const float* seed_real, const float* seed_imag, int64_t begin,
                                int64_t end, REAL* const* g) {
    const int64_t S = c->state_count;
    const int64_t E = c->event_count;
    const cplx zero = {LIT(0.0), LIT(0.0)};
    cplx* traj = (cplx*)malloc(sizeof(cplx) * (size_t)(E > 0 ? E : 1) * (size_t)(3 * S));
    cplx* buf = (cplx*)calloc((size_t)(9 * S), sizeof(cplx));
    cplx *plus = buf, *minus = buf + S, *lon = buf + 2 * S;
    cplx *pb = buf + 3 * S, *mb = buf + 4 * S, *zb = buf + 5 * S;
    cplx *ps = buf + 6 * S, *ms = buf + 7 * S, *zs = buf + 8 * S;
#if defined(REAL_IS_FLOAT)
    const REAL pi = 3.14159265358979323846F;
#else
    const REAL pi = 3.14159265358979323846;
#endif
    for (int64_t work = begin; work < end; ++work) {
        const int64_t train = work / c->atom_count;
        const int64_t atom = work % c->atom_count;
        const int64_t ebase = train * E;
        const float* duration = c->duration_s + ebase;
        const float* flip = c->flip_rad + ebase;
        const float* phase = o->phase_rad ? o->phase_rad + ebase : NULL;
        const int64_t out_base = (train * c->atom_count + atom) * c->output_count;
        const REAL t1 = (REAL)c->t1_ms[atom];
        const REAL t2 = (REAL)c->t2_ms[atom];
        const REAL r1 = LIT(1000.0) / t1;
        const REAL r2 = LIT(1000.0) / t2;
        const REAL m0 = tissue(c->m0, atom, LIT(1.0));
        const REAL b1 = tissue(c->b1, atom, LIT(1.0));
        const REAL eff = tissue(c->inversion, atom, LIT(1.0));
        const REAL b1_phase = tissue(o->b1_phase_rad, atom, LIT(0.0));
        const REAL b0 = tissue(o->b0_hz, atom, LIT(0.0));
        for (int64_t s = 0; s < 9 * S; ++s) buf[s] = zero;
        lon[0].re = LIT(1.0);
        /* The forward, as run_forward_complex, recording entry states. */
        for (int64_t e = 0; e < E; ++e) {
            memcpy(traj + e * 3 * S, plus, sizeof(cplx) * (size_t)(3 * S));
            const REAL dt = (REAL)duration[e];
            const REAL e1 = EXP(-r1 * dt);
            const cplx tr = cpolar(EXP(-r2 * dt), -LIT(2.0) * pi * b0 * dt);
            for (int64_t s = 0; s < S; ++s) {
                plus[s] = cmul(plus[s], tr);
                minus[s] = cmul(minus[s], cconj(tr));
                lon[s] = cscale(e1, lon[s]);
            }
            lon[0].re += LIT(1.0) - e1;
            const uint8_t a = c->action[e];
            if (a & A_PRE_SHIFT) shift_complex(plus, minus, S);
            if (c->kind[e] == 1) {
                if (a & A_INVERSION) {
                    for (int64_t s = 0; s < S; ++s) lon[s] = cscale(-eff, lon[s]);
                } else {
                    const REAL phi = (phase ? (REAL)phase[e] : LIT(0.0)) + b1_phase;
                    rotate_complex(plus, minus, lon, S, (REAL)flip[e] * b1, phi);
                }
            }
            if (a & A_POST_SHIFT) shift_complex(plus, minus, S);
            if (a & A_SPOIL_AFTER) {
                for (int64_t s = 0; s < S; ++s) plus[s] = minus[s] = zero;
            } else if (a & A_SHIFT_AFTER) {
                shift_complex(plus, minus, S);
            }
        }
        for (int64_t s = 0; s < 3 * S; ++s) pb[s] = zero;
        REAL gt1 = 0, gt2 = 0, gm0 = 0, gb1 = 0, ginv = 0, gb1p = 0, gb0 = 0;
        for (int64_t e = E - 1; e >= 0; --e) {
            const cplx* slot = traj + e * 3 * S;
            const uint8_t a = c->action[e];
            const REAL dt = (REAL)duration[e];
            const REAL e1 = EXP(-r1 * dt);
            const cplx tr = cpolar(EXP(-r2 * dt), -LIT(2.0) * pi * b0 * dt);
            for (int64_t s = 0; s < S; ++s) {
                ps[s] = cmul(slot[s], tr);
                ms[s] = cmul(slot[S + s], cconj(tr));
                zs[s] = cscale(e1, slot[2 * S + s]);
            }
            zs[0].re += LIT(1.0) - e1;
            if (a & A_PRE_SHIFT) shift_complex(ps, ms, S);
            if (a & A_SPOIL_AFTER) {
                for (int64_t s = 0; s < S; ++s) pb[s] = mb[s] = zero;
            } else if (a & A_SHIFT_AFTER) {
                shift_complex_adjoint(pb, mb, S);
            }
            if (a & A_POST_SHIFT) shift_complex_adjoint(pb, mb, S);
            const REAL ph = phase ? (REAL)phase[e] : LIT(0.0);
            if (c->kind[e] == 1) {
                if (a & A_INVERSION) {
                    for (int64_t s = 0; s < S; ++s) {
                        ginv -= zb[s].re * zs[s].re + zb[s].im * zs[s].im;
                        zb[s] = cscale(-eff, zb[s]);
                    }
                } else {
                    REAL ga = 0, gp = 0;
                    rotate_complex_adjoint(pb, mb, zb, ps, ms, zs, S, (REAL)flip[e] * b1,
                                           ph + b1_phase, &ga, &gp);
                    g[7][ebase + e] += ga * b1;
                    gb1 += ga * (REAL)flip[e];
                    g[9][ebase + e] += gp;
                    gb1p += gp;
                }
            } else if (c->kind[e] == 2 && (a & A_RECORD)) {
                const int64_t idx = out_base + c->output_index[e];
                const cplx sd = {(REAL)seed_real[idx], (REAL)seed_imag[idx]};
                const cplx d = cpolar(LIT(1.0), -ph);
                const cplx v = cmul(cscale(m0, ps[0]), d);
                const cplx fd = cmul(ps[0], d);
                gm0 += sd.re * fd.re + sd.im * fd.im;
                /* dv/dph = -i v. */
                g[9][ebase + e] += sd.re * v.im - sd.im * v.re;
                pb[0] = cadd(pb[0], cscale(m0, cmul(cconj(d), sd)));
            }
            if (a & A_PRE_SHIFT) shift_complex_adjoint(pb, mb, S);
            /* Relaxation and turn: y = T x on F+, conj(T) x on F-, e1 x + (1 - e1)
             * on Z. With A+ = sum conj(pb) slot+, A- = sum conj(mb) slot-:
             * dL/dlog(e2) = Re(A+ T) + Re(A- conj T), dL/doff = -Im(A+ T) +
             * Im(A- conj T), dL/dlog(e1) = e1 (Re sum conj(zb) slotz - Re zb0). */
            cplx ap = zero, am = zero;
            REAL az = LIT(0.0);
            for (int64_t s = 0; s < S; ++s) {
                ap = cadd(ap, cmul(cconj(pb[s]), slot[s]));
                am = cadd(am, cmul(cconj(mb[s]), slot[S + s]));
                az += zb[s].re * slot[2 * S + s].re + zb[s].im * slot[2 * S + s].im;
            }
            const cplx apt = cmul(ap, tr), amt = cmul(am, cconj(tr));
            const REAL g2 = apt.re + amt.re;
            const REAL goff = -apt.im + amt.im;
            const REAL g1 = e1 * (az - zb[0].re);
            gt2 += g2 * dt * (LIT(1000.0) / (t2 * t2));
            gt1 += g1 * dt * (LIT(1000.0) / (t1 * t1));
            gb0 += goff * (-LIT(2.0) * pi * dt);
            g[8][ebase + e] += -r2 * g2 - r1 * g1 + goff * (-LIT(2.0) * pi * b0);
            for (int64_t s = 0; s < S; ++s) {
                pb[s] = cmul(pb[s], cconj(tr));
                mb[s] = cmul(mb[s], tr);
                zb[s] = cscale(e1, zb[s]);
            }
        }
        const REAL tissue_g[7] = {gt1, gt2, gm0, gb1, ginv, gb1p, gb0};
        for (int k = 0; k < 7; ++k) g[k][atom] += tissue_g[k];
    }
    free(buf);
    free(traj);
}

/* ---- threaded drivers -------------------------------------------------- */

typedef struct {
    const oracle_case* c;
    const oracle_direction* d;
    const oracle_offaxis* o;
    int64_t begin, end;
    REAL* out_real;
    REAL* out_imag;
} job;

static void* forward_job(void* p) {
    job* j = (job*)p;
    run_forward(j->c, j->begin, j->end, j->out_real, j->out_imag);
    return NULL;
}

static void* tangent_job(void* p) {
    job* j = (job*)p;
    run_tangent(j->c, j->d, j->begin, j->end, j->out_real, j->out_imag);
    return NULL;
}

static void* tangent_lanes_job(void* p) {
    job* j = (job*)p;
    run_tangent_lanes(j->c, j->d, j->begin, j->end, j->out_real, j->out_imag);
    return NULL;
}

static void* complex_job(void* p) {
    job* j = (job*)p;
    run_forward_complex(j->c, j->o, j->begin, j->end, j->out_real, j->out_imag);
    return NULL;
}

static void run_threads_o(void* (*fn)(void*), const oracle_case* c, const oracle_direction* d,
                          const oracle_offaxis* o, REAL* out_real, REAL* out_imag, int threads);

static void run_threads(void* (*fn)(void*), const oracle_case* c,
                        const oracle_direction* d, REAL* out_real, REAL* out_imag,
                        int threads) {
    run_threads_o(fn, c, d, NULL, out_real, out_imag, threads);
}

static void run_threads_o(void* (*fn)(void*), const oracle_case* c, const oracle_direction* d,
                          const oracle_offaxis* o, REAL* out_real, REAL* out_imag, int threads) {
    const int64_t work = fn == tangent_lanes_job
                             ? c->train_count * ((c->atom_count + OLANES - 1) / OLANES)
                             : c->atom_count * c->train_count;
    if (threads < 1) threads = 1;
    if (threads > 256) threads = 256;
    if (work < threads) threads = work > 0 ? (int)work : 1;
    pthread_t tid[256];
    job jobs[256];
    const int64_t block = (work + threads - 1) / threads;
    for (int t = 0; t < threads; ++t) {
        jobs[t].c = c;
        jobs[t].d = d;
        jobs[t].o = o;
        jobs[t].begin = t * block < work ? t * block : work;
        jobs[t].end = (t + 1) * block < work ? (t + 1) * block : work;
        jobs[t].out_real = out_real;
        jobs[t].out_imag = out_imag;
    }
    if (threads == 1) {
        fn(&jobs[0]);
        return;
    }
    for (int t = 0; t < threads; ++t) pthread_create(&tid[t], NULL, fn, &jobs[t]);
    for (int t = 0; t < threads; ++t) pthread_join(tid[t], NULL);
}

/* Output planes are (train_count, atom_count, output_count) in REAL. */
void NAME(oracle_forward)(const oracle_case* c, REAL* out_real, REAL* out_imag,
                          int threads) {
    run_threads(forward_job, c, NULL, out_real, out_imag, threads);
}

void NAME(oracle_tangent)(const oracle_case* c, const oracle_direction* d,
                          REAL* out_real, REAL* out_imag, int threads) {
    run_threads(tangent_job, c, d, out_real, out_imag, threads);
}

/* The tangent in the reference's eight-atom lane layout (run_tangent_lanes);
 * its threads split the (train, atom block) items into contiguous ranges, as
 * the reference's pool does (_epg_cpu.cpp:10910-10921). */
void NAME(oracle_tangent_lanes)(const oracle_case* c, const oracle_direction* d,
                                REAL* out_real, REAL* out_imag, int threads) {
    run_threads(tangent_lanes_job, c, d, out_real, out_imag, threads);
}

void NAME(oracle_forward_complex)(const oracle_case* c, const oracle_offaxis* o,
                                  REAL* out_real, REAL* out_imag, int threads) {
    run_threads_o(complex_job, c, NULL, o, out_real, out_imag, threads);
}

/* Single-threaded forward over reverse; value[7] and curve[7] (t1, t2, m0,
 * b1, inversion per atom; flip, duration per train and event) must be
 * zeroed by the caller. */
void NAME(oracle_second)(const oracle_case* c, const oracle_direction* d, const float* seed_imag,
                         REAL* const* value, REAL* const* curve) {
    run_second(c, d, seed_imag, 0, c->atom_count * c->train_count, value, curve);
}

/* Single-threaded complex adjoint; g[10] (t1, t2, m0, b1, inversion, b1
 * phase, b0 per atom; flip, duration, phase per train and event) must be
 * zeroed by the caller. */
void NAME(oracle_adjoint_complex)(const oracle_case* c, const oracle_offaxis* o,
                                  const float* seed_real, const float* seed_imag,
                                  REAL* const* g) {
    run_adjoint_complex(c, o, seed_real, seed_imag, 0, c->atom_count * c->train_count, g);
}

/* Single-threaded adjoint; gradient arrays must be zeroed by the caller. */
void NAME(oracle_adjoint)(const oracle_case* c, const float* seed_imag,
                          REAL* g_t1, REAL* g_t2, REAL* g_m0, REAL* g_b1, REAL* g_inv,
                          REAL* g_flip, REAL* g_duration) {
    run_adjoint(c, seed_imag, 0, c->atom_count * c->train_count,
                g_t1, g_t2, g_m0, g_b1, g_inv, g_flip, g_duration);
}
