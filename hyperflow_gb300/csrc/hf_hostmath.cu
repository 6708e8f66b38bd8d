// Host build of the kernels' arithmetic (hf_device.cuh, hf_intdiv.cuh) for the CPU test
// suite: the same source the GPU kernels compile, exposed as plain C functions so the
// tests can compare it with the oracle and with IEEE division / sqrt without a GPU.
// Built as a separate library (libhf_hostmath.so); the product library does not use it.
#include <cstdint>

#include "hf_device.cuh"

extern "C" {

void hm_div(const double* a, const double* b, double* out, int64_t n) {
    for (int64_t i = 0; i < n; ++i) out[i] = hf::div_rn(a[i], b[i]);
}

void hm_half(const double* x, double* out, int64_t n) {
    for (int64_t i = 0; i < n; ++i) out[i] = hf::half(x[i]);
}

void hm_sqrt(const double* x, double* out, int64_t n) {
    for (int64_t i = 0; i < n; ++i) out[i] = hf::sqrt_rn(x[i]);
}

int hm_hllc(double gamma, const double* ul, const double* ur, int dir, double* f) {
    return dir == 0 ? hf::hllc_cons<0>(gamma, gamma - 1.0, ul, ur, f)
                    : hf::hllc_cons<1>(gamma, gamma - 1.0, ul, ur, f);
}

double hm_limiter(int kind, double r) { return kind == 0 ? hf::limiter<0>(r) : hf::limiter<1>(r); }

double hm_slope(int kind, double um, double u0, double up) {
    return kind == 0 ? hf::slope<0>(um, u0, up) : hf::slope<1>(um, u0, up);
}

// bit 0 lt(a,b), 1 le0(a), 2 ge0(a), 3 abs_le(a, 1e-6); out[0] smin, out[1] smax, out[2] nmax(|b|, a)
int hm_compare(double a, double b, double* out) {
    out[0] = hf::smin(a, b);
    out[1] = hf::smax(a, b);
    out[2] = hf::nmax(std::fabs(b), a);
    return (hf::lt(a, b) ? 1 : 0) | (hf::le0(a) ? 2 : 0) | (hf::ge0(a) ? 4 : 0) |
           (hf::abs_le(a, 1e-6) ? 8 : 0);
}

void hm_wave_terms(double gamma, const double* u, double* s2) {
    hf::wave_terms(gamma, gamma - 1.0, u[0], u[1], u[2], u[3], s2[0], s2[1]);
}

}  // extern "C"
