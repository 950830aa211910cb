// visco.hpp -- FP64 set-up of the generalized Zener body shared by the host
// medium set-up (host.cpp) and the device medium set-up (medium.cuh).
//
// relaxation_times and constq_zeta follow src/shared/m_fdtool.f90:691-812;
// relaxed_chi is the phase-velocity ratio of relaxed_medium
// (src/swpc_3d/m_medium.f90:231-271), chi = 1 / Re(1 / sqrt(1 - c tau)),
// written in closed form: for z = a + ib with a > 0,
//   Re(1 / sqrt(z)) = sqrt((|z| + a) / 2) / |z|,
// so that host and device evaluate the same sequence of correctly rounded
// operations and give the same bits.
#pragma once
#include <cmath>

namespace swpc {
namespace visco {

constexpr double PI = 3.14159265358979323846;

inline void relaxation_times(int nm, double fmin, double fmax, double* ts) {
    double oa = 2 * PI * fmin, ob = 2 * PI * fmax;
    if (nm == 1) { ts[0] = 1.0 / std::sqrt(oa * ob); return; }
    for (int m = 0; m < nm; ++m) ts[m] = 1.0 / (oa * std::pow(ob / oa, (double)m / (nm - 1)));
}

inline double constq_zeta(int nm, double fmin, double fmax, const double* ts) {
    double oa = 2 * PI * fmin, ob = 2 * PI * fmax, i0 = 0, i1 = 0, i2 = 0;
    for (int m = 0; m < nm; ++m) {
        double t = ts[m];
        i0 += (std::log(1 + ob * ob * t * t) - std::log(1 + oa * oa * t * t)) / (2 * t);
        i1 += ((std::atan(ob * t) - ob * t / (1 + ob * ob * t * t)) - (std::atan(oa * t) - oa * t / (1 + oa * oa * t * t))) / (2 * t);
    }
    for (int a = 0; a < nm - 1; ++a)
        for (int b = a + 1; b < nm; ++b) {
            double w1 = std::atan(ob * ts[a]) / ts[a] - std::atan(ob * ts[b]) / ts[b];
            double w2 = std::atan(oa * ts[a]) / ts[a] - std::atan(oa * ts[b]) / ts[b];
            i2 += ts[a] * ts[b] / (ts[b] * ts[b] - ts[a] * ts[a]) * (w1 - w2);
        }
    return i0 / (i1 + 2 * i2);
}

// c = (1/nm) sum_m i w tau_m / (1 - i w tau_m), w = 2 pi fq_ref
// (m_medium.f90:241-249): real and imaginary parts
inline void zener_c(int nm, double fq_ref, const double* ts, double& cr, double& ci) {
    const double om = 2 * PI * fq_ref;
    cr = 0;
    ci = 0;
    for (int m = 0; m < nm; ++m) {
        const double x = om * ts[m], d = 1 + x * x;
        cr += -(x * x) / d;
        ci += x / d;
    }
    cr /= nm;
    ci /= nm;
}

// chi of relaxed_medium for the tau-method ratio tau (host; the build uses
// -ffp-contract=off, so no operation is fused)
inline double relaxed_chi(double cr, double ci, double tau) {
    const double a = 1.0 - cr * tau, b = 0.0 - ci * tau;
    const double az = std::sqrt(a * a + b * b);
    return az / std::sqrt((az + a) * 0.5);
}

// The relaxed moduli from the unrelaxed ones (m_medium.f90:250-268): with
// rc = 1 / chi^2 of mu (tau = taus) and of lambda + 2 mu (tau = taup),
//   mu' = mu rc_mu,  lambda' = (lambda + 2 mu) rc_lam - 2 mu'.
inline double relax_factor(double cr, double ci, double tau) {
    const double c = relaxed_chi(cr, ci, tau);
    return 1.0 / (c * c);
}

}  // namespace visco
}  // namespace swpc
