// The state machine of a mixed-precision CG solve whose partial sums every
// participant holds bit-identically (the persistent whole-grid solve of
// mixed_grid.cu, the one-CTA-per-system batched solve of batched.cu): the
// transitions of mixed.cu's k_mx_init / mx_finish / mx_step /
// k_mx_true_residual, advanced by one thread and read by the others after a
// barrier.
//
// A step's totals arrive as float-float values and its scalars are FP32: the
// thread that advances the state does it while every other thread of its CTA
// waits at the next barrier, and on GB300's narrow FP64 pipe each FP64
// operation or conversion on that path costs tens of cycles (in the cluster
// engine, which has the same state machine, FP64 state cost 1 us per step).
// FP64 is kept for the reliable updates: the true residual and the norms of b.
#pragma once

#include "ffsum.cuh"
#include "internal.hpp"

namespace simall {

struct MixedState {
    double b_norm;   // ||b||
    double bnorm;    // max(||b||, 1e-30), the stop test's denominator
    double last;     // the last true relative residual
    double rr_true;  // |b - A x|^2 at the last reliable update
    FF rz;           // r.r of the current step
    float sigma0, rmax, t0;  // iterated residual norm after the last update, its running maximum, true residual then
    float alpha_f, beta_f;   // the step's FP32 coefficients
    float smin;              // smallest iterated residual norm since the last update
    int stall;              // steps since smin was last lowered
    int iter, updates, need, done, result, status, par;
    bool fresh;   // the next step forms p from a replaced residual
    bool update;  // the step just finished asks for a reliable update

    __device__ void start(double sbb, double bb, double tol, int max_iter)
    {
        const double bn = sqrt(bb);
        b_norm = bn;
        bnorm = bn > 1e-30 ? bn : 1e-30;
        rz = FF{static_cast<float>(sbb), 0.0f};
        sigma0 = sqrtf(static_cast<float>(sbb));
        rmax = sigma0;
        smin = sigma0;
        stall = 0;
        const double tr = bn / bnorm;
        t0 = static_cast<float>(tr);
        last = tr;
        rr_true = bb;
        alpha_f = beta_f = 0.0f;
        iter = updates = result = 0;
        need = 2;  // the first (FRESH) step is not counted as an update
        done = 0;
        status = SIMALL_OK;
        par = 1;   // the first step forms p = r (beta = 0) at parity 1
        fresh = true;
        update = false;
        if (tr < tol) {
            done = 1;  // b == 0: x = 0 is exact
        } else if (max_iter <= 0) {
            done = 1;
            result = max_iter;
        }
    }

    // alpha and beta are used in FP32, so they are divided in FP32;
    // |r - alpha q|^2, which cancels, is formed in float-float with the FP32
    // alpha the step will use.  t = {p.q, q.q, r.r, r.q}, renormalised.
    __device__ void coefficients(const FF (&t)[4])
    {
        const FF pq = t[0], qq = t[1], rr = t[2], rq = t[3];
        if (!(pq.hi > 0.0f) || !(rr.hi > 0.0f)) {  // not SPD in FP32, or exact breakdown
            status = SIMALL_ERR_BREAKDOWN;
            need = 1;
            alpha_f = beta_f = 0.0f;
        } else {
            alpha_f = __fdiv_rn(rr.hi, pq.hi);
            const FF next = ff_next_rr(rr, qq, rq, alpha_f);
            beta_f = __fdiv_rn(next.hi > 0.0f ? next.hi : 0.0f, rr.hi);
        }
    }

    // tolf, deltaf: the tolerance and the update trigger as floats
    __device__ void finish_step(const FF (&t)[4], float tolf, float deltaf, int max_iter)
    {
        const FF rr = t[2];
        if (fresh) {
            rz = rr;
            sigma0 = sqrtf(rr.hi);
            rmax = sigma0;
            smin = sigma0;
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
        // the trigger and the estimate (the stop test itself is the FP64 true
        // residual of the reliable update this asks for)
        const float sigma = sqrtf(rr.hi);
        const float est = t0 * __fdiv_rn(sigma, sigma0);
        if (sigma < smin) {
            smin = sigma;
            stall = 0;
        } else {
            ++stall;
        }
        if (need || sigma < deltaf * rmax || est < tolf || iter >= max_iter || stall >= kMixedStallSteps) {
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
        t0 = static_cast<float>(tt);
        update = false;
        if (tt < tol) {
            done = 1;
            result = iter;
        } else if (iter >= max_iter || status == SIMALL_ERR_BREAKDOWN) {
            done = 1;
            result = iter >= max_iter ? max_iter : iter;
        } else {
            beta_f = static_cast<float>(a[1] / ff_double(rz));
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
        s->rz = ff_double(rz);
        s->alpha = alpha_f;
        s->beta = beta_f;
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
