// The state machine of a mixed-precision CG solve whose partial sums every
// participant holds bit-identically (the persistent whole-grid solve of
// mixed_grid.cu, the one-CTA-per-system batched solve of batched.cu): the
// transitions of mixed.cu's k_mx_init / mx_finish / mx_step /
// k_mx_true_residual, advanced by one thread and read by the others after a
// barrier.
#pragma once

#include "internal.hpp"

namespace simall {

struct MixedState {
    double b_norm;  // ||b||
    double bnorm;   // max(||b||, 1e-30), the stop test's denominator
    double rz, sigma0, rmax, t0, last, rr_true, alpha, beta;
    float alpha_f, beta_f;  // the step's FP32 coefficients
    float smin;             // smallest iterated residual norm since the last update
    int stall;              // steps since smin was last lowered
    int iter, updates, need, done, result, status, par;
    bool fresh;   // the next step forms p from a replaced residual
    bool update;  // the step just finished asks for a reliable update

    __device__ void start(double sbb, double bb, double tol, int max_iter)
    {
        const double bn = sqrt(bb);
        b_norm = bn;
        bnorm = bn > 1e-30 ? bn : 1e-30;
        rz = sbb;
        sigma0 = sqrt(sbb);
        rmax = sigma0;
        smin = static_cast<float>(sigma0);
        stall = 0;
        t0 = bn / bnorm;
        last = t0;
        rr_true = bb;
        alpha = beta = 0.0;
        alpha_f = beta_f = 0.0f;
        iter = updates = result = 0;
        need = 2;  // the first (FRESH) step is not counted as an update
        done = 0;
        status = SIMALL_OK;
        par = 1;   // the first step forms p = r (beta = 0) at parity 1
        fresh = true;
        update = false;
        if (t0 < tol) {
            done = 1;  // b == 0: x = 0 is exact
        } else if (max_iter <= 0) {
            done = 1;
            result = max_iter;
        }
    }

    // alpha and beta are used in FP32, so they are divided in FP32: GB300's
    // FP64 divide and square root are long chains on a narrow pipe, and this
    // runs on the critical path of every step.  |r - alpha q|^2, which
    // cancels, is formed in FP64 with the FP32 alpha the step will use.
    __device__ void coefficients(const double (&t)[4])
    {
        const double pq = t[0], qq = t[1], rr = t[2], rq = t[3];
        if (!(pq > 0.0) || !(rr > 0.0)) {  // not SPD in FP32, or exact breakdown
            status = SIMALL_ERR_BREAKDOWN;
            need = 1;
            alpha_f = beta_f = 0.0f;
        } else {
            alpha_f = __fdiv_rn(static_cast<float>(rr), static_cast<float>(pq));
            const double a = alpha_f;
            const double next = rr - 2.0 * a * rq + a * a * qq;
            beta_f = __fdiv_rn(static_cast<float>(next > 0.0 ? next : 0.0), static_cast<float>(rr));
        }
        alpha = alpha_f;
        beta = beta_f;
    }

    __device__ void finish_step(const double (&t)[4], double tol, double delta, int max_iter)
    {
        const double rr = t[2];
        if (fresh) {
            rz = rr;
            sigma0 = sqrtf(static_cast<float>(rr));
            rmax = sigma0;
            smin = static_cast<float>(sigma0);
            stall = 0;
            if (need == 1)
                ++updates;
            need = 0;
            coefficients(t);
            fresh = false;
            par ^= 1;
            update = need == 1;
            return;
        }
        ++iter;
        // the trigger and the estimate in FP32 (the same reason as above)
        const float sigma = sqrtf(static_cast<float>(rr));
        const float est = static_cast<float>(t0) * __fdiv_rn(sigma, static_cast<float>(sigma0));
        last = est;
        if (sigma < smin) {
            smin = sigma;
            stall = 0;
        } else {
            ++stall;
        }
        if (need || sigma < static_cast<float>(delta) * static_cast<float>(rmax) || est < static_cast<float>(tol) ||
            iter >= max_iter || stall >= kMixedStallSteps) {
            need = 1;  // fold, true residual, replacement, then a FRESH step at this parity
            update = true;
            return;
        }
        if (sigma > rmax)
            rmax = sigma;
        rz = rr;
        coefficients(t);
        par ^= 1;
        update = need == 1;
    }

    // a = {|b - A x|^2, |S (b - A x)|^2 of the FP32 replacement}
    __device__ void finish_update(const double (&a)[2], double tol, int max_iter)
    {
        rr_true = a[0];
        const double tt = sqrt(a[0]) / bnorm;
        last = tt;
        t0 = tt;
        update = false;
        if (tt < tol) {
            done = 1;
            result = iter;
        } else if (iter >= max_iter || status == SIMALL_ERR_BREAKDOWN) {
            done = 1;
            result = iter >= max_iter ? max_iter : iter;
        } else {
            beta = a[1] / rz;
            beta_f = static_cast<float>(beta);
            fresh = true;
        }
    }

    __device__ void stop(int why)
    {
        status = why;
        done = 1;
        result = iter;
    }

    __device__ void publish(SolveScalars *s, bool ok) const
    {
        s->rz = rz;
        s->alpha = alpha;
        s->beta = beta;
        s->rr = rr_true;
        s->bnorm = bnorm;
        s->last = last;
        s->sigma0 = sigma0;
        s->t0 = t0;
        s->rmax = rmax;
        s->iter = iter;
        s->result = result;
        s->done = done;
        s->status = ok ? status : SIMALL_ERR_TIMEOUT;
        s->need_update = 0;
        s->updates = updates;
    }
};

}  // namespace simall
