// Test program (built and run by tests/test_adjoint_host.py): the reverse
// passes of sgx_adjoint.cuh against central differences of the forward
// functions, and the separated right-hand side against the reference
// grouping of the oracle (geodesic_oracle.hpp), all in double on the host.
// Prints three worst relative errors: rhs_vjp7, step_vjp state and constants,
// and the separated-vs-reference right-hand side.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <random>

#include "sgx_adjoint.cuh"
#include "geodesic_oracle.hpp"

using namespace sgxa;

int main() {
    std::mt19937 rng(3);
    std::uniform_real_distribution<double> U(0, 1);
    double w_rhs = 0, w_state = 0, w_const = 0, w_same = 0;
    for (int t = 0; t < 2000; ++t) {
        double th = 0.2 + 2.7 * U(rng);
        if (t % 7 == 0) th = std::asin((U(rng) < 0.5 ? -1 : 1) * (0.03 + 0.15 * U(rng)));  // pole damping active
        double y[8] = {3 + 27 * U(rng), th, 6.28 * U(rng), -3 + 6 * U(rng), -4 + 8 * U(rng), 3 * U(rng),
                       std::sin(th), std::cos(th)};
        const double E = 0.8 + 0.4 * U(rng), L = -5 + 10 * U(rng), a = 0.99 * U(rng), M = 1;
        const double h = 0.05 + 0.3 * U(rng), e = 1e-6;
        const bool fade = (t % 2) == 0;
        // right-hand side: w . J against central differences
        {
            double w[7], gy[8], gc[3] = {0, 0, 0};
            for (double& x : w) x = -1 + 2 * U(rng);
            rhs_vjp7(y, E, L, a, M, w, gy, gc);
            const int idx[5] = {0, 3, 4, 6, 7};
            for (int k = 0; k < 8; ++k) {
                double yp[8], ym[8];
                std::copy(y, y + 8, yp);
                std::copy(y, y + 8, ym);
                double Ep = E, Em = E, Lp = L, Lm = L, ap = a, am = a;
                if (k < 5) {
                    yp[idx[k]] += e;
                    ym[idx[k]] -= e;
                } else if (k == 5) {
                    Ep += e;
                    Em -= e;
                } else if (k == 6) {
                    Lp += e;
                    Lm -= e;
                } else {
                    ap += e;
                    am -= e;
                }
                double dp[7], dm[7];
                rhs7(yp, Ep, Lp, ap, M, dp);
                rhs7(ym, Em, Lm, am, M, dm);
                double fd = 0;
                for (int i = 0; i < 7; ++i) fd += w[i] * (dp[i] - dm[i]) / (2 * e);
                const double got = k < 5 ? gy[idx[k]] : gc[k - 5];
                w_rhs = std::max(w_rhs, std::fabs(got - fd) / std::max(1.0, std::fabs(fd)));
            }
        }
        // one step: lam . J against central differences
        {
            double lam[8], lv[8], gc[3] = {0, 0, 0};
            for (double& x : lam) x = -1 + 2 * U(rng);
            std::copy(lam, lam + 8, lv);
            step_vjp(y, E, L, a, M, h, fade, lv, gc);
            for (int k = 0; k < 11; ++k) {
                double yp[8], ym[8];
                std::copy(y, y + 8, yp);
                std::copy(y, y + 8, ym);
                double Ep = E, Em = E, Lp = L, Lm = L, ap = a, am = a;
                if (k < 8) {
                    yp[k] += e;
                    ym[k] -= e;
                } else if (k == 8) {
                    Ep += e;
                    Em -= e;
                } else if (k == 9) {
                    Lp += e;
                    Lm -= e;
                } else {
                    ap += e;
                    am -= e;
                }
                double op[8], om[8];
                step(yp, Ep, Lp, ap, M, h, fade, op);
                step(ym, Em, Lm, am, M, h, fade, om);
                double fd = 0;
                for (int i = 0; i < 8; ++i) fd += lam[i] * (op[i] - om[i]) / (2 * e);
                const double got = k < 8 ? lv[k] : gc[k - 8];
                const double rel = std::fabs(got - fd) / std::max(1.0, std::fabs(fd));
                if (k < 8) w_state = std::max(w_state, rel);
                else w_const = std::max(w_const, rel);
            }
        }
        // the separated form against the reference grouping
        {
            double d[7];
            rhs7(y, E, L, a, M, d);
            const oracle::KState<double> s{0, y[0], y[1], y[2], y[3], y[4]};
            const oracle::KConst<double> c{E, L, 0, a, M};
            const oracle::KState<double> o = oracle::kerr_rhs(s, c);
            const double ref[5] = {o.r, o.theta, o.phi, o.p_r, o.p_theta};
            const double sc = 1e-3 * (std::fabs(o.r) + std::fabs(o.p_r) + 1);
            for (int i = 0; i < 5; ++i)
                w_same = std::max(w_same, std::fabs(d[i] - ref[i]) / (std::fabs(ref[i]) + sc));
            w_same = std::max(w_same, std::fabs(d[5] - y[7] * o.theta) / (std::fabs(o.theta) + sc));
            w_same = std::max(w_same, std::fabs(d[6] + y[6] * o.theta) / (std::fabs(o.theta) + sc));
        }
    }
    std::printf("%.3e %.3e %.3e %.3e\n", w_rhs, w_state, w_const, w_same);
    return 0;
}
