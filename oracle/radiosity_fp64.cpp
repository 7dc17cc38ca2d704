// ORACLE -- test infrastructure, not product code.
//
// FP64 Jacobi iteration of the radiosity bounce for many right-hand sides,
// the checker of the GPU gather (ltrg_GatherSolve). It restates the
// reference's bounce (Int_RDBounce, lighter.cpp:767-797: every linked pair
// passes out * diffuse * area * f of one element to the other, `total`
// accumulates, `out` becomes what was received) in double precision:
//
//   B_0 = E,   B_k = E + K B_{k-1},   K_ij = f_ij * area_j * albedo_j(r mod 3)
//
// which after k sweeps equals the reference's total = sum_{m<=k} K^m E.
// f_ij is recomputed in double from the patch positions and normals with the
// reference's expression (lighter.cpp:743-747: f = dA dB / (|d|^4 pi)); which
// pairs are linked (the visibility bits) is taken from the FP32 pass, as the
// nonzero entries of `mask_G` (n x n, row-major). Rows run on `threads`
// threads; the result does not depend on the thread count.
#include <math.h>
#include <stdint.h>
#include <string.h>

#include <algorithm>
#include <atomic>
#include <thread>
#include <vector>

typedef uint32_t u32;

extern "C" __attribute__((visibility("default"))) void orc_gather_jacobi_f64(
    u32 n, u32 R, const float* pos3, const float* nrm3, const float* area, const float* mask_G, const float* albedo,
    const float* E, int bounces, double* out, int threads)
{
    std::vector<double> P(3 * (size_t) n), N(3 * (size_t) n);
    for (u32 i = 0; i < n; ++i) {
        double x = nrm3[3 * i], y = nrm3[3 * i + 1], z = nrm3[3 * i + 2];
        double l = sqrt(x * x + y * y + z * z);
        if (l > 0) { x /= l; y /= l; z /= l; }
        N[3 * i] = x; N[3 * i + 1] = y; N[3 * i + 2] = z;
        for (int c = 0; c < 3; ++c) P[3 * i + c] = pos3[3 * i + c];
    }
    std::vector<double> B((size_t) n * R), X((size_t) n * R);
    for (size_t t = 0; t < (size_t) n * R; ++t) B[t] = E[t];
    const double pi = 3.14159265358979323846;
    auto row = [&](u32 i, std::vector<double>& acc) {
        std::fill(acc.begin(), acc.end(), 0.0);
        const float* m = mask_G + (size_t) i * n;
        const double* ap = &P[3 * (size_t) i];
        const double* an = &N[3 * (size_t) i];
        for (u32 j = 0; j < n; ++j) {
            if (m[j] == 0.0f) continue;
            const double* bp = &P[3 * (size_t) j];
            const double* bn = &N[3 * (size_t) j];
            double dx = bp[0] - ap[0], dy = bp[1] - ap[1], dz = bp[2] - ap[2];
            double dA = an[0] * dx + an[1] * dy + an[2] * dz;
            double dB = -(bn[0] * dx + bn[1] * dy + bn[2] * dz);
            double l2 = dx * dx + dy * dy + dz * dz;
            double g = dA * dB / (l2 * l2 * pi) * (double) area[j];
            const double* xj = &X[(size_t) j * R];
            for (u32 r = 0; r < R; ++r) acc[r] += g * xj[r];
        }
    };
    for (int b = 0; b < bounces; ++b) {
        for (u32 j = 0; j < n; ++j)
            for (u32 r = 0; r < R; ++r) X[(size_t) j * R + r] = (double) albedo[3 * j + r % 3] * B[(size_t) j * R + r];
        std::atomic<u32> next(0);
        int nt = std::max(1, std::min<int>(threads, (int) n));
        std::vector<std::thread> pool;
        for (int t = 0; t < nt; ++t)
            pool.emplace_back([&]() {
                std::vector<double> acc(R);
                for (;;) {
                    u32 i = next.fetch_add(1);
                    if (i >= n) break;
                    row(i, acc);
                    for (u32 r = 0; r < R; ++r) B[(size_t) i * R + r] = (double) E[(size_t) i * R + r] + acc[r];
                }
            });
        for (auto& th : pool) th.join();
    }
    memcpy(out, B.data(), sizeof(double) * (size_t) n * R);
}
