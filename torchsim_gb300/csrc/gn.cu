// Per-voxel Levenberg-Marquardt in FP64 on the device: the step and the
// accept/damping decision of the reference's GaussNewton under a TrustRegion
// (recon/_gauss_newton.py:475-631, TrustRegion 366-415), one thread per
// voxel, over normal equations that the GN evaluation sweep reduced.
//
// Variables are the unconstrained images of the bounded properties
// (_bounds.py:77-199): a two-sided bound maps through a sigmoid, a one-sided
// one through softplus, and the Jacobian is widened by the chain factor. The
// reference solves the damped step as the augmented least-squares problem
// [J^T; sqrt(a) I] d = [r; 0] in FP32 (direct, _gauss_newton.py:247-307);
// here its normal equations (J^T J + a I) d = -J^T r are solved by a 3x3
// Cholesky factorisation in FP64.
#include <math.h>

#include "tsg_internal.h"

namespace tsg {
namespace {

constexpr double kTiny = 1.1754943508222875e-38;  // smallest normal float

__device__ __forceinline__ double sigmoid(double u) { return 1.0 / (1.0 + exp(-u)); }

__device__ __forceinline__ double softplus(double u) {
    return u > 30.0 ? u : log1p(exp(u));
}

__device__ __forceinline__ void to_natural(const tsg_gn_config& c, const double* u, double* x) {
    for (int k = 0; k < 3; ++k) {
        const double lo = c.low[k], hi = c.high[k];
        const bool has_lo = isfinite(lo), has_hi = isfinite(hi);
        if (has_lo && has_hi)
            x[k] = lo + (hi - lo) * sigmoid(u[k]);
        else if (has_lo)
            x[k] = lo + softplus(u[k]);
        else if (has_hi)
            x[k] = hi - softplus(-u[k]);
        else
            x[k] = u[k];
    }
}

__device__ __forceinline__ void widen(const tsg_gn_config& c, const double* u, double* w) {
    for (int k = 0; k < 3; ++k) {
        const double lo = c.low[k], hi = c.high[k];
        const bool has_lo = isfinite(lo), has_hi = isfinite(hi);
        if (has_lo && has_hi) {
            const double s = sigmoid(u[k]);
            w[k] = (hi - lo) * s * (1.0 - s);
        } else if (has_lo) {
            w[k] = sigmoid(u[k]);
        } else if (has_hi) {
            w[k] = sigmoid(-u[k]);
        } else {
            w[k] = 1.0;
        }
    }
}

// Free-variable normal equations from natural ones: A_f = W A W, g_f = W g.
__device__ __forceinline__ void free_system(const double* ne, const double* w, double A[3][3],
                                            double* g) {
    const double a11 = ne[1], a12 = ne[2], a13 = ne[3], a22 = ne[4], a23 = ne[5], a33 = ne[6];
    A[0][0] = w[0] * w[0] * a11;
    A[0][1] = A[1][0] = w[0] * w[1] * a12;
    A[0][2] = A[2][0] = w[0] * w[2] * a13;
    A[1][1] = w[1] * w[1] * a22;
    A[1][2] = A[2][1] = w[1] * w[2] * a23;
    A[2][2] = w[2] * w[2] * a33;
    // ne holds sum dv*(v + y): the gradient of the cost in s = -v is J_s^T r
    // with J_s = -dv and r = -(v + y), i.e. the same sum.
    g[0] = w[0] * ne[7];
    g[1] = w[1] * ne[8];
    g[2] = w[2] * ne[9];
}

// Solves (A + lambda I) d = -g; false when the matrix is not positive definite.
__device__ bool damped_solve(const double A[3][3], const double* g, double lambda, double* d) {
    double L[3][3] = {};
    double M[3][3];
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) M[i][j] = A[i][j] + (i == j ? lambda : 0.0);
    for (int j = 0; j < 3; ++j) {
        double s = M[j][j];
        for (int k = 0; k < j; ++k) s -= L[j][k] * L[j][k];
        if (!(s > 0.0) || !isfinite(s)) return false;
        L[j][j] = sqrt(s);
        for (int i = j + 1; i < 3; ++i) {
            double t = M[i][j];
            for (int k = 0; k < j; ++k) t -= L[i][k] * L[j][k];
            L[i][j] = t / L[j][j];
        }
    }
    double y[3];
    for (int i = 0; i < 3; ++i) {
        double t = -g[i];
        for (int k = 0; k < i; ++k) t -= L[i][k] * y[k];
        y[i] = t / L[i][i];
    }
    for (int i = 2; i >= 0; --i) {
        double t = y[i];
        for (int k = i + 1; k < 3; ++k) t -= L[k][i] * d[k];
        d[i] = t / L[i][i];
    }
    return isfinite(d[0]) && isfinite(d[1]) && isfinite(d[2]);
}

__global__ void gn_step_kernel(tsg_gn_state s, int64_t n, tsg_gn_config c) {
    const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int status = s.status[i];
    if (status == TSG_GN_DONE) return;
    double u[3] = {s.u[3 * i], s.u[3 * i + 1], s.u[3 * i + 2]};
    double cand[3] = {u[0], u[1], u[2]};
    if (status == TSG_GN_LIVE) {
        const double* ne = s.normal + 10 * i;
        double w[3], A[3][3], g[3];
        widen(c, u, w);
        free_system(ne, w, A, g);
        // A voxel whose gradient is flat is finished before it steps
        // (_gauss_newton.py:560-565).
        const double gmax = fmax(fabs(g[0]), fmax(fabs(g[1]), fabs(g[2])));
        if (gmax < c.gradient_tolerance) {
            s.status[i] = TSG_GN_DONE;
            return;
        }
        const double lambda = s.damping[i];
        double d[3];
        const bool ok = damped_solve(A, g, lambda, d);
        int flags = 0;
        if (!ok) {
            flags |= 2;  // singular: the step is not taken
            d[0] = d[1] = d[2] = nan("");
        }
        double pred = 0.0, walked = 0.0, norm_u = 0.0;
        for (int k = 0; k < 3; ++k) {
            pred += d[k] * (lambda * d[k] - g[k]);
            walked += d[k] * d[k];
            norm_u += u[k] * u[k];
            cand[k] = u[k] + d[k];
        }
        walked = sqrt(walked);
        norm_u = sqrt(norm_u);
        if (ok && walked < c.step_tolerance * (norm_u + c.step_tolerance)) flags |= 1;
        s.predicted[i] = pred;
        s.flags[i] = flags;
    }
    for (int k = 0; k < 3; ++k) s.cand[3 * i + k] = cand[k];
    double x[3];
    to_natural(c, cand, x);
    s.t1[i] = float(x[0]);
    s.t2[i] = float(x[1]);
    s.m0[i] = float(x[2]);
}

__global__ void gn_judge_kernel(tsg_gn_state s, int64_t n, tsg_gn_config c) {
    const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int status = s.status[i];
    if (status == TSG_GN_DONE) return;
    const double* tr = s.trial + 10 * i;
    double* ne = s.normal + 10 * i;
    if (status == TSG_GN_FIRST) {
        // The first evaluation is taken as it stands and sets the damping
        // from the curvature there (TrustRegion.begin, :389-393).
        for (int k = 0; k < 10; ++k) ne[k] = tr[k];
        s.cost[i] = tr[0];
        double u[3] = {s.u[3 * i], s.u[3 * i + 1], s.u[3 * i + 2]};
        double w[3], A[3][3], g[3];
        widen(c, u, w);
        free_system(ne, w, A, g);
        s.damping[i] = c.tau * fmax(A[0][0], fmax(A[1][1], A[2][2]));
        s.rising[i] = 2.0;
        s.iterations[i] = 0;
        s.status[i] = TSG_GN_LIVE;
        return;
    }
    const int flags = s.flags[i];
    const bool singular = (flags & 2) != 0;
    const bool is_short = (flags & 1) != 0;
    const double pred = s.predicted[i];
    const double cost = s.cost[i];
    const double trial_cost = tr[0];
    const double gain = pred > 0.0 ? (cost - trial_cost) / fmax(pred, kTiny) : 0.0;
    const bool better = gain > 0.0 && !singular;
    // Nielsen's update (TrustRegion.judge, :395-411).
    const double lambda = s.damping[i];
    const double rising = s.rising[i];
    const double q = 2.0 * gain - 1.0;
    const double lowered = lambda * fmax(1.0 - q * q * q, 1.0 / 3.0);
    s.damping[i] = better ? lowered : lambda * rising;
    s.rising[i] = better ? 2.0 : rising * 2.0;
    if (better) {
        for (int k = 0; k < 3; ++k) s.u[3 * i + k] = s.cand[3 * i + k];
        for (int k = 0; k < 10; ++k) ne[k] = tr[k];
        s.cost[i] = trial_cost;
    }
    const int it = s.iterations[i] + 1;
    s.iterations[i] = it;
    if (is_short && !singular) {
        s.status[i] = TSG_GN_DONE;
    } else if (it >= c.max_iterations) {
        s.status[i] = TSG_GN_DONE;
        s.flags[i] = flags | 4;  // stopped by the step limit: unconverged
    }
}

__global__ void gn_natural_kernel(const double* u, int64_t n, tsg_gn_config c, float* out) {
    const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= n) return;
    double uu[3] = {u[3 * i], u[3 * i + 1], u[3 * i + 2]};
    double x[3];
    to_natural(c, uu, x);
    for (int k = 0; k < 3; ++k) out[3 * i + k] = float(x[k]);
}

bool valid(const tsg_gn_state* s) {
    return s && s->u && s->cand && s->cost && s->normal && s->trial && s->damping && s->rising &&
           s->predicted && s->status && s->flags && s->iterations && s->t1 && s->t2 && s->m0;
}

}  // namespace
}  // namespace tsg

using namespace tsg;

extern "C" int tsg_gn_step(const tsg_gn_state* state, int64_t voxel_count,
                           const tsg_gn_config* config, void* stream) {
    if (voxel_count < 0 || !config || (voxel_count > 0 && !valid(state)))
        return fail(TSG_ERR_ARGUMENT, "invalid Gauss-Newton state");
    if (voxel_count == 0) return TSG_OK;
    gn_step_kernel<<<unsigned((voxel_count + 127) / 128), 128, 0, static_cast<cudaStream_t>(stream)>>>(
        *state, voxel_count, *config);
    TSG_CUDA(cudaGetLastError());
    return TSG_OK;
}

extern "C" int tsg_gn_judge(const tsg_gn_state* state, int64_t voxel_count,
                            const tsg_gn_config* config, void* stream) {
    if (voxel_count < 0 || !config || (voxel_count > 0 && !valid(state)))
        return fail(TSG_ERR_ARGUMENT, "invalid Gauss-Newton state");
    if (voxel_count == 0) return TSG_OK;
    gn_judge_kernel<<<unsigned((voxel_count + 127) / 128), 128, 0, static_cast<cudaStream_t>(stream)>>>(
        *state, voxel_count, *config);
    TSG_CUDA(cudaGetLastError());
    return TSG_OK;
}

extern "C" int tsg_gn_natural(const double* free_variables, int64_t voxel_count,
                              const tsg_gn_config* config, float* natural, void* stream) {
    if (voxel_count < 0 || !config || (voxel_count > 0 && (!free_variables || !natural)))
        return fail(TSG_ERR_ARGUMENT, "invalid arguments");
    if (voxel_count == 0) return TSG_OK;
    gn_natural_kernel<<<unsigned((voxel_count + 127) / 128), 128, 0, static_cast<cudaStream_t>(stream)>>>(
        free_variables, voxel_count, *config, natural);
    TSG_CUDA(cudaGetLastError());
    return TSG_OK;
}
