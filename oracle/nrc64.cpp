// Test infrastructure only: NOT part of the product.
//
// CPU oracle of the neural radiance cache network (the product's kernels are
// raycer_gb300/csrc/nrc.cu): input encoding, forward pass, gradient of the
// relative L2 loss and one Adam step. The reference has no counterpart (its
// PathTracer::traceRecursive, src/Raytracing/Tracers/PathTracer.cpp:30-75,
// always recurses to maxPathLength), so this restates the network's own
// definition:
//
//   features (128): for axis a, k = 0..11: sin, cos(pi 2^k u_a),
//                   u = (x_a - lo_a) * inv_a; for axis a, k = 0..3:
//                   sin, cos(pi 2^k (w_a + 1) / 2); normal; albedo; 1; 0 pad
//   h1..h4 = relu(W_l h_{l-1}), z = W5 h4 (rows 0..2), p = exp(z)
//   loss   = sum_{i,c} (p - y)^2 / (p^2 + 0.01) / (3 n), the denominator
//            held constant for the gradient
//   Adam   m = b1 m + (1-b1) g, v = b2 v + (1-b2) g^2,
//          w -= lr (m / (1-b1^t)) / (sqrt(v / (1-b2^t)) + eps)   (float32)
//
// emulate = 0: everything in float64 with the float32 master weights.
// emulate = 1: the kernels' rounding points in float64 arithmetic: BF16
// (round to nearest even) weights, features, activations, loss gradient and
// back-propagated gradients; float32 for the position scaling and the loss
// gradient's formula.

#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>

#include <omp.h>

namespace
{

constexpr int kIn = 128;
constexpr int kH = 64;
constexpr int kParams = 20992;
constexpr int kW1 = 0, kW2 = 8192, kW3 = 12288, kW4 = 16384, kW5 = 20480;
constexpr double kPi = 3.14159265358979323846;

double bf16(double x)
{
    float f = float(x);
    uint32_t b;
    std::memcpy(&b, &f, 4);
    if ((b & 0x7f800000u) == 0x7f800000u)
        return x;
    b += 0x7fffu + ((b >> 16) & 1u);
    b &= 0xffff0000u;
    std::memcpy(&f, &b, 4);
    return double(f);
}

void features(const float* q, const float* lo, const float* inv, int emulate, double* out)
{
    for (int a = 0; a < 3; ++a)
    {
        double u;
        if (emulate)
        {
            volatile float d = q[a] - lo[a];
            volatile float m = d * inv[a];
            u = double(m);
        }
        else
            u = (double(q[a]) - double(lo[a])) * double(inv[a]);
        for (int k = 0; k < 12; ++k)
        {
            double x = std::ldexp(u, k);
            out[a * 24 + 2 * k] = std::sin(kPi * x);
            out[a * 24 + 2 * k + 1] = std::cos(kPi * x);
        }
    }
    for (int a = 0; a < 3; ++a)
    {
        double u;
        if (emulate)
        {
            volatile float s = q[3 + a] + 1.0f;
            volatile float m = 0.5f * s;
            u = double(m);
        }
        else
            u = 0.5 * (double(q[3 + a]) + 1.0);
        for (int k = 0; k < 4; ++k)
        {
            double x = std::ldexp(u, k);
            out[72 + a * 8 + 2 * k] = std::sin(kPi * x);
            out[72 + a * 8 + 2 * k + 1] = std::cos(kPi * x);
        }
    }
    for (int c = 0; c < 6; ++c)
        out[96 + c] = double(q[6 + c]);
    out[102] = 1.0;
    for (int c = 103; c < kIn; ++c)
        out[c] = 0.0;
    if (emulate)
        for (int c = 0; c < kIn; ++c)
            out[c] = bf16(out[c]);
}

std::vector<double> weights(const float* params, int emulate)
{
    std::vector<double> w(kParams);
    for (int i = 0; i < kParams; ++i)
        w[size_t(i)] = emulate ? bf16(double(params[i])) : double(params[i]);
    return w;
}

struct Activations
{
    double h[5][kIn];  // h[0] = features (128), h[1..4] hidden (64)
    double z[3];
    double p[3];
};

void forward(const std::vector<double>& w, const double* f, int emulate, Activations& a)
{
    std::memcpy(a.h[0], f, sizeof(double) * kIn);
    const int offs[4] = { kW1, kW2, kW3, kW4 };
    for (int l = 0; l < 4; ++l)
    {
        const int nin = l == 0 ? kIn : kH;
        const double* W = w.data() + offs[l];
        for (int o = 0; o < kH; ++o)
        {
            double s = 0.0;
            for (int i = 0; i < nin; ++i)
                s += W[o * nin + i] * a.h[l][i];
            s = s > 0.0 ? s : 0.0;
            a.h[l + 1][o] = emulate ? bf16(s) : s;
        }
    }
    for (int o = 0; o < 3; ++o)
    {
        double s = 0.0;
        for (int i = 0; i < kH; ++i)
            s += w[size_t(kW5 + o * kH + i)] * a.h[4][i];
        a.z[o] = s;
        a.p[o] = std::exp(s);
    }
}

}  // namespace

extern "C" {

void or_nrc_features(const float* queries, int64_t n, const float* lo, const float* inv, int emulate, double* out)
{
#pragma omp parallel for schedule(static)
    for (int64_t r = 0; r < n; ++r)
        features(queries + r * 12, lo, inv, emulate, out + r * kIn);
}

void or_nrc_forward(const float* params, const float* queries, int64_t n, const float* lo, const float* inv,
                    int emulate, double* rgb)
{
    const std::vector<double> w = weights(params, emulate);
#pragma omp parallel for schedule(static)
    for (int64_t r = 0; r < n; ++r)
    {
        double f[kIn];
        features(queries + r * 12, lo, inv, emulate, f);
        Activations a;
        forward(w, f, emulate, a);
        for (int c = 0; c < 3; ++c)
            rgb[r * 3 + c] = a.p[c];
    }
}

// Loss with the denominator p0^2 + 0.01 taken from `den_pred` (n x 3), or
// from the prediction itself when den_pred is null.
double or_nrc_loss(const float* params, const float* queries, const float* targets, int64_t n, const float* lo,
                   const float* inv, int emulate, const double* den_pred)
{
    const std::vector<double> w = weights(params, emulate);
    double total = 0.0;
#pragma omp parallel for schedule(static) reduction(+ : total)
    for (int64_t r = 0; r < n; ++r)
    {
        double f[kIn];
        features(queries + r * 12, lo, inv, emulate, f);
        Activations a;
        forward(w, f, emulate, a);
        for (int c = 0; c < 3; ++c)
        {
            double p0 = den_pred ? den_pred[r * 3 + c] : a.p[c];
            double d = a.p[c] - double(targets[r * 3 + c]);
            total += d * d / (p0 * p0 + 0.01);
        }
    }
    return total / (3.0 * double(n));
}

// Gradient of the loss (grad: kParams doubles, padding rows 3..7 zero); returns the loss.
double or_nrc_gradient(const float* params, const float* queries, const float* targets, int64_t n, const float* lo,
                       const float* inv, int emulate, double* grad)
{
    const std::vector<double> w = weights(params, emulate);
    const int threads = omp_get_max_threads();
    std::vector<std::vector<double>> part(size_t(threads), std::vector<double>(kParams, 0.0));
    std::vector<double> lossPart(size_t(threads), 0.0);
    const double scale = 1.0 / (3.0 * double(n));
    const float scalef = 1.0f / (float(n) * 3.0f);
#pragma omp parallel
    {
        const int tid = omp_get_thread_num();
        std::vector<double>& g = part[size_t(tid)];
#pragma omp for schedule(static)
        for (int64_t r = 0; r < n; ++r)
        {
            double f[kIn];
            features(queries + r * 12, lo, inv, emulate, f);
            Activations a;
            forward(w, f, emulate, a);
            double dz[kH];
            double dzOut[3];
            for (int c = 0; c < 3; ++c)
            {
                const double p = a.p[c];
                const double y = double(targets[r * 3 + c]);
                const double den = p * p + 0.01;
                lossPart[size_t(tid)] += (p - y) * (p - y) / den * scale;
                if (emulate)
                {
                    const float pf = float(p), yf = targets[r * 3 + c];
                    volatile float denf = pf * pf + 0.01f;
                    volatile float diff = pf - yf;
                    volatile float t = 2.0f * diff;
                    t = t / denf;
                    t = t * scalef;
                    t = t * pf;
                    dzOut[c] = bf16(double(t));
                }
                else
                    dzOut[c] = 2.0 * (p - y) / den * scale * p;
            }
            // output layer
            for (int o = 0; o < 3; ++o)
                for (int i = 0; i < kH; ++i)
                    g[size_t(kW5 + o * kH + i)] += dzOut[o] * a.h[4][i];
            for (int i = 0; i < kH; ++i)
            {
                double s = 0.0;
                for (int o = 0; o < 3; ++o)
                    s += dzOut[o] * w[size_t(kW5 + o * kH + i)];
                s = a.h[4][i] > 0.0 ? s : 0.0;
                dz[i] = emulate ? bf16(s) : s;
            }
            // hidden layers 4, 3, 2 (W4, W3, W2) and the input layer (W1)
            const int offs[4] = { kW1, kW2, kW3, kW4 };
            for (int l = 3; l >= 0; --l)
            {
                const int nin = l == 0 ? kIn : kH;
                const double* W = w.data() + offs[l];
                for (int o = 0; o < kH; ++o)
                    for (int i = 0; i < nin; ++i)
                        g[size_t(offs[l] + o * nin + i)] += dz[o] * a.h[l][i];
                if (l == 0)
                    break;
                double nd[kH];
                for (int i = 0; i < kH; ++i)
                {
                    double s = 0.0;
                    for (int o = 0; o < kH; ++o)
                        s += dz[o] * W[o * nin + i];
                    s = a.h[l][i] > 0.0 ? s : 0.0;
                    nd[i] = emulate ? bf16(s) : s;
                }
                std::memcpy(dz, nd, sizeof(nd));
            }
        }
    }
    double loss = 0.0;
    for (int i = 0; i < kParams; ++i)
    {
        double s = 0.0;
        for (int t = 0; t < threads; ++t)
            s += part[size_t(t)][size_t(i)];
        grad[i] = s;
    }
    for (int t = 0; t < threads; ++t)
        loss += lossPart[size_t(t)];
    return loss;
}

// One Adam step in float32 (t >= 1 is the step number after this update).
void or_nrc_adam(float* master, float* m, float* v, const float* grad, int64_t t, float lr, float b1, float b2,
                 float eps)
{
    const float b1p = float(std::pow(double(b1), double(t)));
    const float b2p = float(std::pow(double(b2), double(t)));
    for (int i = 0; i < kParams; ++i)
    {
        volatile float g = grad[i];
        volatile float mi = b1 * m[i] + (1.0f - b1) * g;
        volatile float gg = g * g;
        volatile float vi = b2 * v[i] + (1.0f - b2) * gg;
        m[i] = mi;
        v[i] = vi;
        volatile float mh = mi / (1.0f - b1p);
        volatile float vh = vi / (1.0f - b2p);
        volatile float den = std::sqrt(vh) + eps;
        master[i] = master[i] - lr * mh / den;
    }
}

}  // extern "C"
