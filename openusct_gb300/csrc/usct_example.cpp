// usct_example.cpp -- using libusct_gb300 from plain C++ (no Python).
//
// The counterpart of the reference's native example for its C++ core
// (software/core/example_main.cpp): build a small 2D model with a slow flaw,
// record a full-matrix capture with a ring of elements, then evaluate the L2
// and the GCN misfit and their gradients from a homogeneous start model, and
// print checksums.  It calls the host-pointer entry points, whose argument
// lists are those of uap::forward_fmc / uap::misfit_and_gradient
// (libuap.hpp:109,169).
//
// Build (after the library is built):
//   g++ -O2 -std=c++14 -I include openusct_gb300/csrc/usct_example.cpp \
//       -L openusct_gb300 -lusct_gb300 -Wl,-rpath,$PWD/openusct_gb300 -o usct_example
#include <cmath>
#include <cstdio>
#include <vector>

#include "usct_gb300.h"

namespace {

const double kPi = 3.14159265358979323846;

int fail(const char* what, int code) {
    std::fprintf(stderr, "%s failed (%d): %s\n", what, code, usct_last_error());
    return 1;
}

}  // namespace

int main() {
    const int n = 48;
    const int dims[2] = {n, n};
    const double h = 1.0e-3, dt = 1.4e-7, f0 = 0.35e6;
    const int nt = 320;
    const size_t cells = (size_t)n * n;

    // Ricker source, peak at t = 1/f0
    std::vector<double> wavelet(nt);
    for (int i = 0; i < nt; ++i) {
        const double u = kPi * f0 * (i * dt - 1.0 / f0);
        wavelet[i] = (1.0 - 2.0 * u * u) * std::exp(-u * u);
    }

    // 2950 m/s background, 2500 m/s disc of radius 5 mm at (0.6, 0.45) of the domain
    const double L = (n - 1) * h;
    std::vector<double> m_true(cells), m0(cells, 1.0 / (2950.0 * 2950.0));
    for (int iy = 0; iy < n; ++iy)
        for (int ix = 0; ix < n; ++ix) {
            const double dx = ix * h - 0.60 * L, dy = iy * h - 0.45 * L;
            const double c = (dx * dx + dy * dy <= 0.005 * 0.005) ? 2500.0 : 2950.0;
            m_true[(size_t)iy * n + ix] = 1.0 / (c * c);
        }

    // 16 elements on a ring of radius 18 mm, as row-major linear indices
    const int ne = 16;
    std::vector<int> elem(ne);
    for (int k = 0; k < ne; ++k) {
        const double a = 2.0 * kPi * k / ne;
        const int ix = (int)std::lround((0.5 * L + 0.018 * std::cos(a)) / h);
        const int iy = (int)std::lround((0.5 * L + 0.018 * std::sin(a)) / h);
        elem[k] = iy * n + ix;
    }

    std::vector<double> data((size_t)ne * nt * ne);
    int rc = usct_forward_fmc(m_true.data(), dims, 2, h, dt, nt, elem.data(), ne, elem.data(), ne,
                              wavelet.data(), data.data());
    if (rc != USCT_OK) return fail("usct_forward_fmc", rc);
    double sd = 0.0;
    for (double v : data) sd += std::fabs(v);
    std::printf("forward_sum_abs=%.9e\n", sd);

    std::vector<double> grad(cells);
    double J = 0.0;
    rc = usct_misfit_and_gradient(m0.data(), dims, 2, h, dt, nt, elem.data(), ne, elem.data(), ne,
                                  wavelet.data(), data.data(), grad.data(), &J);
    if (rc != USCT_OK) return fail("usct_misfit_and_gradient", rc);
    double sg = 0.0;
    for (double v : grad) sg += std::fabs(v);
    std::printf("l2_J=%.9e\nl2_grad_sum_abs=%.9e\n", J, sg);

    rc = usct_misfit_and_gradient_mt(m0.data(), dims, 2, h, dt, nt, elem.data(), ne, elem.data(),
                                     ne, wavelet.data(), data.data(), grad.data(), 1, &J);
    if (rc != USCT_OK) return fail("usct_misfit_and_gradient_mt", rc);
    sg = 0.0;
    for (double v : grad) sg += std::fabs(v);
    std::printf("gcn_J=%.9e\ngcn_grad_sum_abs=%.9e\n", J, sg);
    std::printf("usct_example OK\n");
    return 0;
}
