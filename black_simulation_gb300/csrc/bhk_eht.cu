// bhk_eht.cu -- eht::render on the GPU: the shadow and the 230 GHz synchrotron image of a hot, thick
// flow, one ray per thread, in FP64.
//
// The image is a sum over the integrator's steps (each step adds g^3 S (1 - e^-dtau) dimmed by the
// depth in front), so it depends on the steps taken: the kernel restates eht::traceRay's own loop
// (src/eht.cpp:260-319) -- Bardeen launch at r = 1000 M, kerr::photonStepSize at tolerance 0.05
// (0.02 inside 60 M), kerr::stepMino, enforceConstraints then normalizeAngles, capture below
// r_+(1 + 1e-4), exit back past 1010 M, emission gathered inside 60 M until the optical depth
// passes 30 -- and the flow and emission models it calls (src/eht.cpp:99-258). This translation
// unit is compiled without FMA contraction, so its FP64 arithmetic follows the reference's C++.
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "bhk_device.cuh"
#include "bhk_internal.h"

namespace bhk {
namespace eht {

// Physical constants, CGS (src/eht.cpp:25-34: CODATA values).
constexpr double kElectronCharge = 4.80320425e-10;
constexpr double kElectronMass = 9.1093837015e-28;
constexpr double kProtonMass = 1.67262192369e-24;
constexpr double kLight = 2.99792458e10;
constexpr double kBoltzmann = 1.380649e-16;
constexpr double kPlanck = 6.62607015e-27;
constexpr double kSolarLengthCm = 1.476625e5;
constexpr double kJansky = 1e-23;
constexpr double kMicroarcsecond = kPi / 180.0 / 3600.0 / 1e6;
// The image's geometry (src/eht.cpp:14-16).
constexpr double kStartRadius = 1000.0, kLightRadius = 60.0, kMaxDepth = 30.0;

// Boyer-Lindquist metric components the flow needs (src/eht.cpp:19-27).
struct BL {
    double gtt, gtp, gpp, grr;
};
__device__ __forceinline__ BL metric_bl(double a, double r, double theta) {
    const double sn = sin(theta);
    const double s2 = sn * sn, c2 = 1.0 - s2;
    const double sigma = r * r + a * a * c2, delta = r * r - 2.0 * r + a * a;
    const double A = (r * r + a * a) * (r * r + a * a) - a * a * delta * s2;
    return {-(1.0 - 2.0 * r / sigma), -2.0 * a * r * s2 / sigma, A * s2 / sigma, sigma / delta};
}

// Circular equatorial orbit constants, prograde (src/kerr.cpp:308-319).
__device__ __forceinline__ void circular_orbit(double a, double r, double* E, double* L) {
    const double sr = sqrt(r), r32 = r * sr;
    const double den = pow(r, 0.75) * sqrt(r32 - 3.0 * sr + 2.0 * a);
    *E = (r32 - 2.0 * sr + a) / den;
    *L = (r * r - 2.0 * a * sr + a * a) / den;
}

// |u^r| of the plunge from the ISCO at r inside it (src/eht.cpp:192-200).
__device__ __forceinline__ double plunge_speed(double a, double r, double isco) {
    double E, L;
    circular_orbit(a, isco, &E, &L);
    const double delta = r * r - 2.0 * r + a * a, x = L - a * E;
    const double P = E * (r * r + a * a) - a * L;
    return sqrt(fmax(P * P - delta * (r * r + x * x), 0.0)) / (r * r);
}

// Modified Bessel functions from the polynomial approximations of Abramowitz & Stegun, Handbook of
// Mathematical Functions, 9.8.1-9.8.8 (the coefficients are the published ones; the reference uses
// the same approximations). horner(c, y) = c[0] + y (c[1] + y (c[2] + ...)).
template <int N>
__device__ __forceinline__ double horner(const double (&c)[N], double y) {
    double acc = c[N - 1];
#pragma unroll
    for (int k = N - 2; k >= 0; --k) acc = c[k] + y * acc;
    return acc;
}

__device__ __forceinline__ double bessel_i0(double x) {  // A&S 9.8.1 (|x| < 3.75), 9.8.2
    constexpr double small[7] = {1.0, 3.5156229, 3.0899424, 1.2067492, 0.2659732, 0.360768e-1, 0.45813e-2};
    constexpr double large[9] = {0.39894228, 0.1328592e-1, 0.225319e-2, -0.157565e-2, 0.916281e-2,
                                 -0.2057706e-1, 0.2635537e-1, -0.1647633e-1, 0.392377e-2};
    const double ax = fabs(x);
    if (ax < 3.75) {
        const double t = x / 3.75;
        return horner(small, t * t);
    }
    return (exp(ax) / sqrt(ax)) * horner(large, 3.75 / ax);
}

__device__ __forceinline__ double bessel_i1(double x) {  // A&S 9.8.3 (|x| < 3.75), 9.8.4
    constexpr double small[7] = {0.5, 0.87890594, 0.51498869, 0.15084934, 0.2658733e-1, 0.301532e-2, 0.32411e-3};
    constexpr double large[9] = {0.39894228, -0.3988024e-1, -0.362018e-2, 0.163801e-2, -0.1031555e-1,
                                 0.2282967e-1, -0.2895312e-1, 0.1787654e-1, -0.420059e-2};
    const double ax = fabs(x);
    double r;
    if (ax < 3.75) {
        const double t = x / 3.75;
        r = ax * horner(small, t * t);
    } else {
        r = horner(large, 3.75 / ax) * exp(ax) / sqrt(ax);
    }
    return x < 0.0 ? -r : r;
}

// K0 and K1 times e^x (A&S 9.8.5-9.8.8; for x > 2 the exponential is factored out, so that the
// emissivity forms without underflow in cold gas).
__device__ __forceinline__ double scaled_k0(double x) {
    constexpr double small[7] = {-0.57721566, 0.42278420, 0.23069756, 0.3488590e-1, 0.262698e-2, 0.10750e-3, 0.74e-5};
    constexpr double large[7] = {1.25331414, -0.7832358e-1, 0.2189568e-1, -0.1062446e-1, 0.587872e-2,
                                 -0.251540e-2, 0.53208e-3};
    if (x <= 2.0) return exp(x) * ((-log(x / 2.0) * bessel_i0(x)) + horner(small, x * x / 4.0));
    return (1.0 / sqrt(x)) * horner(large, 2.0 / x);
}

__device__ __forceinline__ double scaled_k1(double x) {
    constexpr double small[7] = {1.0, 0.15443144, -0.67278579, -0.18156897, -0.1919402e-1, -0.110404e-2, -0.4686e-4};
    constexpr double large[7] = {1.25331414, 0.23498619, -0.3655620e-1, 0.1504268e-1, -0.780353e-2, 0.325614e-2,
                                 -0.68245e-3};
    if (x <= 2.0) return exp(x) * ((log(x / 2.0) * bessel_i1(x)) + (1.0 / x) * horner(small, x * x / 4.0));
    return (1.0 / sqrt(x)) * horner(large, 2.0 / x);
}

// K2 = K0 + (2 / x) K1 (the recurrence), scaled by e^x like its parts.
__device__ __forceinline__ double scaled_k2(double x) { return scaled_k0(x) + 2.0 / x * scaled_k1(x); }

// Thermal synchrotron emissivity, Leung, Gammie & Noble (2011) eq. 72 (src/eht.cpp:163-177).
__device__ __forceinline__ double synchrotron_emissivity(double nu, double ne, double thetaE, double B,
                                                         double sinThetaB) {
    if (ne <= 0.0 || thetaE < 0.05 || B <= 0.0 || sinThetaB <= 0.0) return 0.0;
    const double nuC = kElectronCharge * B / (2.0 * kPi * kElectronMass * kLight);
    const double nuS = (2.0 / 9.0) * nuC * thetaE * thetaE * sinThetaB;
    const double X = nu / nuS;
    const double cube = cbrt(X);
    const double shape = sqrt(X) + pow(2.0, 11.0 / 12.0) * pow(X, 1.0 / 6.0);
    const double inv = 1.0 / thetaE;
    const double exponent = inv - cube;
    if (exponent < -700.0) return 0.0;
    return ne * sqrt(2.0) * kPi * kElectronCharge * kElectronCharge * nuS / (3.0 * scaled_k2(inv) * kLight) * shape *
           shape * exp(exponent);
}

__device__ __forceinline__ double planck(double nu, double T) {
    const double x = kPlanck * nu / (kBoltzmann * T);
    return 2.0 * kPlanck * nu * nu * nu / (kLight * kLight) / expm1(x);
}

struct Plasma {
    double ne, Te, B;
};

// The flow after Broderick & Loeb (2006) with a continuity-matched plunge inside the ISCO
// (src/eht.cpp:204-222).
__device__ __forceinline__ Plasma plasma_at(const bhk_eht_flow& f, double r, double theta, double a, double isco,
                                            double rp) {
    const double z = r * cos(theta), rho = fmax(r * sin(theta), 1e-6);
    Plasma p;
    const double h = fmax(f.height, 0.05) * rho;
    double radial = pow(r, -1.1);
    if (r < isco) {
        const double start = fmax(isco - 0.25, 0.5 * (isco + rp));
        if (r < start) {
            const double here = plunge_speed(a, r, isco), there = plunge_speed(a, start, isco);
            if (here > 0.0) radial = fmin(radial, pow(start, -1.1) * (start * start * there) / (r * r * here));
        }
    }
    p.ne = f.n0 * radial * exp(-z * z / (2.0 * h * h));
    p.Te = f.T0 * pow(r, -0.84);
    p.B = sqrt(8.0 * kPi * p.ne * kProtonMass * kLight * kLight / (6.0 * f.beta * r));
    return p;
}

// The gas's 4-velocity (src/eht.cpp:224-255).
__device__ __forceinline__ void flow_velocity(const bhk_eht_flow& f, double a, double r, double theta, double isco,
                                              double u[4]) {
    const BL g = metric_bl(a, r, theta);
    double omega = 0.0, ur = 0.0;
    if (r >= isco) {
        omega = f.keplerian / (pow(r, 1.5) + a);
    } else {
        double E, L;
        circular_orbit(a, isco, &E, &L);
        const double delta = r * r - 2.0 * r + a * a, x = L - a * E;
        const double P = E * (r * r + a * a) - a * L;
        const double R = fmax(P * P - delta * (r * r + x * x), 0.0);
        const double ut = ((r * r + a * a) * P / delta + a * x) / (r * r);
        const double up = (a * P / delta + x) / (r * r);
        omega = up / ut;
        ur = -sqrt(R) / (r * r);
    }
    double denom = g.gtt + 2.0 * omega * g.gtp + omega * omega * g.gpp;
    double num = -1.0 - g.grr * ur * ur;
    if (!(denom < 0.0) || !(num < 0.0)) {
        omega = -g.gtp / g.gpp;
        ur = 0.0;
        denom = g.gtt + 2.0 * omega * g.gtp + omega * omega * g.gpp;
        num = -1.0;
    }
    const double ut = sqrt(num / denom);
    u[0] = ut;
    u[1] = ur;
    u[2] = 0.0;
    u[3] = omega * ut;
}

// eht::traceRay (src/eht.cpp:260-319) for image-plane point (alpha, beta).
__device__ void trace_pixel(const bhk_eht_view& v, const bhk_eht_flow& f, double alpha, double beta, bool with_light,
                            double isco, double rp, double* intensity, bool* captured, int* steps) {
    const double a = v.a;
    const double sinI = sin(v.inclination), cosI = cos(v.inclination);
    const Cons c{1.0, -alpha * sinI, beta * beta + (alpha * alpha - a * a) * cosI * cosI, 0.0};
    St s{};
    s.r = kStartRadius;
    s.theta = fmin(fmax(v.inclination, 1e-4), kPi - 1e-4);
    s.vr = -sqrt(fmax(radial_potential(a, c, s.r), 0.0));
    s.vtheta = (beta > 0.0 ? -1.0 : 1.0) * sqrt(fmax(polar_potential(a, c, s.theta), 0.0));
    const double lengthCm = kSolarLengthCm * v.mass_solar;
    double I = 0.0, depth = 0.0;
    bool cap = false;
    int step = 0;
    for (; step < 40000; ++step) {
        const double tolerance = s.r < kLightRadius ? 0.02 : 0.05;
        const double h = photon_step_size(a, c, s, tolerance);
        const double cb = cos(s.theta);
        const double sigmaBefore = s.r * s.r + a * a * cb * cb;
        step_mino(a, c, s, h);
        enforce_constraints(a, c, s);
        normalize_angles(s);
        if (!isfinite(s.r) || s.r < rp * (1.0 + 1e-4)) {
            cap = true;
            break;
        }
        if (s.r > kStartRadius * 1.01 && s.vr > 0.0) break;
        if (!with_light || s.r > kLightRadius) continue;
        const double ct = cos(s.theta);
        const double sigma = s.r * s.r + a * a * ct * ct;
        const double dLambda = 0.5 * (sigma + sigmaBefore) * h * lengthCm;
        const Plasma pl = plasma_at(f, s.r, s.theta, a, isco, rp);
        double u[4];
        flow_velocity(f, a, s.r, s.theta, isco, u);
        const double delta = s.r * s.r - 2.0 * s.r + a * a;
        const double pr = -s.vr / delta, pth = -s.vtheta;
        const double minusPu = u[0] - c.L * u[3] - pr * u[1] - pth * u[2];
        if (!(minusPu > 0.0)) continue;
        const double g = 1.0 / minusPu;
        const double nuF = v.frequency / g;
        const double thetaE = kBoltzmann * pl.Te / (kElectronMass * kLight * kLight);
        const double j = synchrotron_emissivity(nuF, pl.ne, thetaE, pl.B, f.sin_theta_b);
        if (j <= 0.0) continue;
        const double absorption = j / planck(nuF, pl.Te);
        const double dTau = absorption * dLambda / g;
        const double added = dTau < 1e-6 ? g * g * j * dLambda : g * g * g * (j / absorption) * -expm1(-dTau);
        I += exp(-depth) * added;
        depth += dTau;
        if (depth > kMaxDepth) break;
    }
    *intensity = I;
    *captured = cap;
    *steps = step;
}

// One thread per pixel (grid-stride), the image row-major from beta = +half_width
// (src/eht.cpp:321-347).
__global__ void render_kernel(bhk_eht_view v, bhk_eht_flow f, int with_light, double rp, double isco,
                              double* intensity, uint8_t* shadow, int32_t* steps) {
    const long long n = static_cast<long long>(v.size) * v.size;
    const double pixel = 2.0 * v.half_width / v.size;
    for (long long k = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; k < n;
         k += static_cast<long long>(gridDim.x) * blockDim.x) {
        const int row = static_cast<int>(k / v.size), col = static_cast<int>(k - static_cast<long long>(row) * v.size);
        const double beta = v.half_width - (row + 0.5) * pixel;
        const double alpha = -v.half_width + (col + 0.5) * pixel;
        double I;
        bool cap;
        int st;
        trace_pixel(v, f, alpha, beta, with_light != 0, isco, rp, &I, &cap, &st);
        if (intensity) intensity[k] = I;
        if (shadow) shadow[k] = cap ? 1 : 0;
        if (steps) steps[k] = st;
    }
}

bool valid(const bhk_eht_view* v, const bhk_eht_flow* f) {
    // |a| > 1 (no horizon): eht::traceRay's capture radius r_+ (1 + 1e-4) is then 0 (src/eht.cpp:274-287).
    return v && f && v->size > 0 && v->size <= 16384 && (std::fabs(v->a) < 1.0 || std::fabs(v->a) > 1.0) &&
           v->half_width > 0.0 &&
           v->frequency > 0.0 && v->mass_solar > 0.0 && f->T0 > 0.0 && f->beta > 0.0;
}

}  // namespace eht
}  // namespace bhk

extern "C" {

bhk_status bhk_eht_render(const bhk_eht_view* view, const bhk_eht_flow* flow, int32_t with_light, double* intensity,
                          uint8_t* shadow, int32_t* steps, void* stream) {
    if (!bhk::eht::valid(view, flow)) {
        bhk::set_last_error("bhk_eht_render: invalid view or flow (size 1..16384, finite |a| != 1, positive scales)");
        return BHK_EINVAL;
    }
    const long long n = static_cast<long long>(view->size) * view->size;
    const int block = 128;
    int device = 0, sms = 0;
    if (cudaGetDevice(&device) != cudaSuccess ||
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device) != cudaSuccess || sms <= 0) {
        cudaGetLastError();
        bhk::set_last_error("bhk_eht_render: no usable CUDA device");
        return BHK_ECUDA;
    }
    const int grid = static_cast<int>(std::min<long long>((n + block - 1) / block, 16LL * sms));
    // Horizon and prograde ISCO once on the host (past |a| = 1 the ISCO is a 4000-point search).
    const double rp = bhk::horizon_radius(view->a), isco = bhk::isco_radius(view->a, true);
    bhk::eht::render_kernel<<<grid, block, 0, static_cast<cudaStream_t>(stream)>>>(*view, *flow, with_light, rp, isco,
                                                                                    intensity, shadow, steps);
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) {
        bhk::set_last_error(std::string("bhk_eht_render: ") + cudaGetErrorString(e));
        return BHK_ECUDA;
    }
    return BHK_OK;
}

// eht::flux (src/eht.cpp:348-353) of a host image: Jy for a source whose M subtends theta_g_uas.
double bhk_eht_flux(const double* intensity, int32_t size, double half_width, double theta_g_uas) {
    if (!intensity || size <= 0) return 0.0;
    const double pixel = 2.0 * half_width / size;
    const double solid = std::pow(pixel * theta_g_uas * bhk::eht::kMicroarcsecond, 2.0);
    double sum = 0.0;
    for (long long k = 0; k < static_cast<long long>(size) * size; ++k) sum += intensity[k];
    return sum * solid / bhk::eht::kJansky;
}

// eht::calibrate (src/eht.cpp:437-460): the density n0 that gives target_jy, by a secant
// iteration in log n0 on 48-pixel renders (on the GPU). Synchronous.
bhk_status bhk_eht_calibrate(const bhk_eht_view* view, const bhk_eht_flow* flow, double target_jy,
                             double theta_g_uas, double* n0_out) {
    if (!bhk::eht::valid(view, flow) || !n0_out || !(target_jy > 0.0)) {
        bhk::set_last_error("bhk_eht_calibrate: invalid arguments");
        return BHK_EINVAL;
    }
    bhk_eht_view small = *view;
    small.size = 48;
    bhk_eht_flow fl = *flow;
    const size_t n = 48 * 48;
    double* d = nullptr;
    if (cudaMalloc(&d, n * sizeof(double)) != cudaSuccess) return BHK_ENOMEM;
    std::vector<double> h(n);
    bhk_status st = BHK_OK;
    auto flux_at = [&](double n0) {
        fl.n0 = n0;
        if (st != BHK_OK) return 0.0;
        st = bhk_eht_render(&small, &fl, 1, d, nullptr, nullptr, nullptr);
        if (st == BHK_OK && cudaMemcpy(h.data(), d, n * sizeof(double), cudaMemcpyDeviceToHost) != cudaSuccess) {
            bhk::set_last_error("bhk_eht_calibrate: copy failed");
            st = BHK_ECUDA;
        }
        return st == BHK_OK ? bhk_eht_flux(h.data(), 48, small.half_width, theta_g_uas) : 0.0;
    };
    double n0 = flow->n0, f0 = flux_at(n0);
    for (int k = 0; k < 8 && f0 <= 0.0 && st == BHK_OK; ++k) f0 = flux_at(n0 *= 10.0);
    double n1 = n0;
    if (f0 > 0.0 && st == BHK_OK) {
        n1 = n0 * target_jy / f0;
        double f1 = flux_at(n1);
        for (int k = 0; k < 8 && st == BHK_OK; ++k) {
            if (f1 <= 0.0 || std::fabs(f1 / target_jy - 1.0) < 0.01) break;
            const double slope = (std::log(f1) - std::log(f0)) / (std::log(n1) - std::log(n0));
            const double next =
                std::exp(std::log(n1) + (std::log(target_jy) - std::log(f1)) / (std::fabs(slope) > 0.05 ? slope : 1.0));
            n0 = n1;
            f0 = f1;
            n1 = std::min(std::max(next, n0 / 30.0), n0 * 30.0);
            f1 = flux_at(n1);
        }
    }
    cudaFree(d);
    if (st != BHK_OK) return st;
    *n0_out = n1;
    return BHK_OK;
}

}  // extern "C"
