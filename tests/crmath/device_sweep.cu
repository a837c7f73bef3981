// The correctly rounded sin / cos / asin / atan2 of avbd_crmath.cuh on the
// GPU against the same functions built for the host and against long-double
// references rounded to float.  Prints one line per function: arguments,
// device-vs-host mismatches, device-vs-reference mismatches.
#include <cuda_runtime.h>

#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <vector>

#include "../../ornis_gb300/csrc/avbd_crmath.cuh"

static float u2f(uint32_t u) { float f; std::memcpy(&f, &u, 4); return f; }
static uint32_t f2u(float f) { uint32_t u; std::memcpy(&u, &f, 4); return u; }
static bool same(float a, float b) { return f2u(a) == f2u(b) || (a != a && b != b); }

__global__ void k_eval(const float* x, const float* y, size_t n, float* s, float* c, float* ss, float* cc, float* as,
                       float* at) {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
        s[i] = avbd::crm::sinf(x[i]);
        c[i] = avbd::crm::cosf(x[i]);
        avbd::crm::sincosf(x[i], &ss[i], &cc[i]);
        as[i] = avbd::crm::asinf(x[i]);
        at[i] = avbd::crm::atan2f(y[i], x[i]);
    }
}

#define CK(e)                                                                     \
    do {                                                                          \
        cudaError_t r_ = (e);                                                     \
        if (r_ != cudaSuccess) {                                                  \
            printf("cuda error %s at %s:%d\n", cudaGetErrorString(r_), __FILE__, __LINE__); \
            return 2;                                                             \
        }                                                                         \
    } while (0)

int main() {
    std::vector<float> xs, ys;
    uint64_t st = 12345;
    auto rnd = [&]() {
        st = st * 6364136223846793005ull + 1442695040888963407ull;
        return (uint32_t)(st >> 32);
    };
    for (uint64_t u = 0; u < (1ull << 32); u += 65537) xs.push_back(u2f((uint32_t)u));
    for (uint32_t u = f2u(0x1p-14f); u < f2u(4.0f); u += 61) xs.push_back(u2f(u));
    for (uint32_t u = f2u(0.5f); u <= f2u(1.0f); u += 17) xs.push_back(u2f(u));
    const float sp[] = {0.0f, -0.0f, INFINITY, -INFINITY, 1.0f, -1.0f, NAN};
    for (float v : sp) xs.push_back(v);
    for (size_t i = 0; i < xs.size(); i++) {
        uint32_t r = rnd();
        float y = i % 3 == 0 ? u2f(r) : (i % 3 == 1 ? xs[i] * u2f(0x3f800000u | (r & 0x7fffffu)) : -xs[i]);
        ys.push_back(y);
    }
    for (float a : sp)
        for (float b : sp) {
            xs.push_back(b);
            ys.push_back(a);
        }
    const size_t n = xs.size();
    float *dx, *dy, *out[6];
    CK(cudaMalloc(&dx, n * 4));
    CK(cudaMalloc(&dy, n * 4));
    for (auto& p : out) CK(cudaMalloc(&p, n * 4));
    CK(cudaMemcpy(dx, xs.data(), n * 4, cudaMemcpyHostToDevice));
    CK(cudaMemcpy(dy, ys.data(), n * 4, cudaMemcpyHostToDevice));
    k_eval<<<1024, 256>>>(dx, dy, n, out[0], out[1], out[2], out[3], out[4], out[5]);
    CK(cudaGetLastError());
    CK(cudaDeviceSynchronize());
    std::vector<float> h[6];
    for (int k = 0; k < 6; k++) {
        h[k].resize(n);
        CK(cudaMemcpy(h[k].data(), out[k], n * 4, cudaMemcpyDeviceToHost));
    }
    long bad_host[5] = {0}, bad_ref[5] = {0};
    const char* names[5] = {"sin", "cos", "sincos", "asin", "atan2"};
    for (size_t i = 0; i < n; i++) {
        float x = xs[i], y = ys[i];
        float hs = avbd::crm::sinf(x), hc = avbd::crm::cosf(x), ha = avbd::crm::asinf(x), ht = avbd::crm::atan2f(y, x);
        float rs = (float)sinl((long double)x), rc = (float)cosl((long double)x);
        float ra = (float)asinl((long double)x), rt = (float)atan2l((long double)y, (long double)x);
        float dev[5] = {h[0][i], h[1][i], h[2][i], h[4][i], h[5][i]};
        float host[5] = {hs, hc, hs, ha, ht}, ref[5] = {rs, rc, rs, ra, rt};
        for (int k = 0; k < 5; k++) {
            if (!same(dev[k], host[k])) bad_host[k]++;
            if (!same(dev[k], ref[k])) {
                if (bad_ref[k] < 3) printf("  %s(%a, %a): device %a, reference %a\n", names[k], x, y, dev[k], ref[k]);
                bad_ref[k]++;
            }
        }
        if (!same(h[3][i], hc)) bad_host[2]++;
    }
    for (int k = 0; k < 5; k++) printf("%s %zu %ld %ld\n", names[k], n, bad_host[k], bad_ref[k]);
    return 0;
}
