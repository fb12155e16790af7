// Substep lengths of LevelSetAdvection::advect under an imposed CFL number.
//
// The reference fixes the CFL number of its substep loop by temporal scheme
// (1/sqrt(3) * {0.3, 0.9, 1.0}, tools/LevelSetAdvect.h:459-463).  A caller
// that wants a smaller CFL number c runs the reference's own advect(tau, tau')
// over greedy intervals: at the start of an interval, with max|v|^2 sampled
// at tau, tau' = tau + c*dx/|v|max (or t1 when that reaches it), and inside
// the interval the reference's loop takes its own substeps
// dt = min(|tau' - t0|, CFL_ref*dx/|v|max) (tools/LevelSetAdvect.h:464-466)
// until t0 reaches tau'.  Normally that is one substep of length
// tau' - tau; when tau + (tau' - tau) rounds short of tau' the reference
// takes a second, short substep, and this clock reproduces it.  Without an
// imposed CFL number (c == 0) the single interval is [t0, t1], which is the
// reference's advect(t0, t1) itself.
#pragma once

#include <cmath>

#include "../../include/gbls.h"

namespace gbls {

// T is the time type: float for the FloatGrid instance (the reference's
// float time), double for the FP64 instance, where the substep lengths
// T(c*dx) / sqrt(T(max |v|^2)) and the time reached are double.
template <class T>
struct CflClockT {
    float t1 = 0.0f;
    bool forward = true;
    float cfl = 0.0f;   // imposed CFL number (0: none)
    float cref = 0.0f;  // the reference's CFL number for the temporal scheme
    float dx = 1.0f;
    bool open = false;  // inside an interval
    T end = T(0.0f);    // the interval's end time
    // how the last substep was set (the adjoint's time-step derivative):
    // limited: CFL_ref*dx/|v|max (else the rest of the interval); opened:
    // the substep opened its interval, whose end is t +- open_lim when
    // end_lim (else t1)
    bool limited = false, opened = false, end_lim = false;
    T open_lim = T(0.0f);

    CflClockT(float t0, float t1_, float cfl_, int temporal, float dx_)
        : t1(t1_), forward(t0 < t1_), cfl(cfl_ > 0.0f ? cfl_ : 0.0f), dx(dx_) {
        cref = (temporal == GBLS_TVD_RK1 ? 0.3f : temporal == GBLS_TVD_RK2 ? 0.9f : 1.0f) / std::sqrt(3.0f);
    }

    bool running(T t) const { return forward ? t < T(t1) : t > T(t1); }

    // Length of the substep that starts at t with max |v|^2 = maxv2 (not
    // approximately zero); 0 ends the loop (an interval that rounds to zero
    // length, where the reference's advect(tau, tau) returns at once).
    T next(T t, T maxv2) {
        opened = false;
        if (!open) {
            end = T(t1);
            end_lim = false;
            if (cfl > 0.0f) {
                const T lim = T(cfl * dx) / std::sqrt(maxv2);
                const T span = std::fabs(T(t1) - t);
                if (lim < span) {
                    end = forward ? t + lim : t - lim;
                    end_lim = true;
                    open_lim = lim;
                }
            }
            if (end - t == T(0.0f)) return T(0.0f);  // math::isZero(time0 - time1)
            open = true;
            opened = true;
        }
        const T span = std::fabs(end - t);
        const T lim = T(cref * dx) / std::sqrt(maxv2);
        limited = lim < span;
        return limited ? lim : span;  // math::Min(dt, CFL*dx/sqrt(maxAbsV))
    }

    // t advanced by the substep dt; closes the interval when t reaches its end.
    void advance(T& t, T dt) {
        t += forward ? dt : -dt;
        if (!(forward ? t < end : t > end)) open = false;
    }
};

using CflClock = CflClockT<float>;

}  // namespace gbls
