// tl_host_numerics.cpp -- see tl_host_numerics.h.  Compiled with
// -ffp-contract=off so the host arithmetic is the same on x86-64 and aarch64.
#include "tl_host_numerics.h"

#include <algorithm>
#include <cmath>
#include <vector>

namespace tl {

int tl_tqli(double *d, double *e, int n) {
    if (n <= 0) return 0;
    // e(:) = eoshift(e(:), 1): sub-diagonal to e[0..n-2]
    for (int i = 0; i + 1 < n; ++i) e[i] = e[i + 1];
    e[n - 1] = 0.0;
    for (int l = 0; l < n; ++l) {
        int sweeps = 0;
        bool again = true;
        while (again) {
            int m = l;
            while (m < n - 1) {
                const double dd = std::fabs(d[m]) + std::fabs(d[m + 1]);
                if (std::fabs(e[m]) + dd == dd) break;
                ++m;
            }
            if (m == l) break;
            if (sweeps == 30) return 1;
            ++sweeps;
            double g = (d[l + 1] - d[l]) / (2.0 * e[l]);
            double r = std::sqrt(g * g + 1.0);
            g = d[m] - d[l] + e[l] / (g + std::copysign(std::fabs(r), g));
            double s = 1.0, c = 1.0, p = 0.0;
            bool deflated = false;
            for (int i = m - 1; i >= l; --i) {
                const double f = s * e[i];
                const double b = c * e[i];
                r = std::sqrt(f * f + g * g);
                e[i + 1] = r;
                if (r == 0.0) {
                    d[i + 1] -= p;
                    e[m] = 0.0;
                    deflated = true;
                    break;
                }
                s = f / r;
                c = g / r;
                g = d[i + 1] - p;
                r = (d[i] - g) * s + 2.0 * c * b;
                p = s * r;
                d[i + 1] = g + p;
                g = c * r - b;
            }
            if (deflated) continue;
            d[l] -= p;
            e[l] = g;
            e[m] = 0.0;
        }
    }
    return 0;
}

int tl_calc_eigenvalues(const double *alphas, const double *betas, int n, double *eigmin,
                        double *eigmax) {
    if (n < 1) return 1;
    std::vector<double> diag(n + 1, 0.0), off(n + 1, 0.0);
    for (int k = 0; k < n; ++k) {
        diag[k] = 1.0 / alphas[k];
        if (k > 0) diag[k] += betas[k - 1] / alphas[k - 1];
        if (k < n - 1) off[k + 1] = std::sqrt(betas[k]) / alphas[k];
    }
    int info = tl_tqli(diag.data(), off.data(), n);
    if (info != 0) return info;
    std::sort(diag.begin(), diag.begin() + n);
    *eigmin = diag[0];
    *eigmax = diag[n - 1];
    if (*eigmin < 0.0 || *eigmax < 0.0) return 1;
    return 0;
}

void tl_calc_ch_coefs(double *alphas, double *betas, double eigmin, double eigmax, double *theta,
                      int n) {
    const double th = (eigmax + eigmin) / 2.0;
    const double delta = (eigmax - eigmin) / 2.0;
    const double sigma = th / delta;
    double rho_old = 1.0 / sigma;
    for (int k = 0; k < n; ++k) {
        const double rho_new = 1.0 / (2.0 * sigma - rho_old);
        alphas[k] = rho_new * rho_old;
        betas[k] = 2.0 * rho_new / delta;
        rho_old = rho_new;
    }
    *theta = th;
}

}  // namespace tl
