// Host side of the FFT engine: factorisation and twiddle tables, cached per
// (device, length) for the life of the process.
#include <math.h>
#include <stdlib.h>
#include <string.h>

#include <algorithm>
#include <map>
#include <mutex>
#include <utility>
#include <vector>

#include "fft.cuh"

namespace {
std::mutex g_mu;
std::map<std::pair<int, int>, FftPlan> g_plans;

// Radix kinds (fft.cuh): 2/3/4/5/7 constant-table registers; 11..37 table
// registers; the other odd primes lane or generic stages, which run first.
// Every stage except 2/3/4/5/7 needs its cos/sin table.
void factor(int n, std::vector<int> &first, std::vector<int> &small) {
    while (n % 4 == 0) { small.push_back(4); n /= 4; }
    while (n % 2 == 0) { small.push_back(2); n /= 2; }
    for (int p : {3, 5, 7})
        while (n % p == 0) { small.push_back(p); n /= p; }
    // a 2 and a 3 become one radix-6 pass
    {
        auto i2 = std::find(small.begin(), small.end(), 2);
        auto i3 = std::find(small.begin(), small.end(), 3);
        if (i2 != small.end() && i3 != small.end()) {
            small.erase(i3);
            *std::find(small.begin(), small.end(), 2) = 6;
        }
    }
    std::vector<int> mid;
    for (int p = 11; (long)p * p <= n; p += 2)
        while (n % p == 0) { (p <= 37 ? mid : first).push_back(p); n /= p; }
    if (n > 1) (n <= 37 ? mid : first).push_back(n);
    // the table-driven odd stages go after the large ones, before the constant radices
    small.insert(small.begin(), mid.begin(), mid.end());
}
// Rader tables of a prime stage R (stage_rader in fft.cuh; g a primitive
// root mod R, 3 for 113 and 7 for 239), appended after its cos/sin table: the
// FFT-M (M = R - 1) of the Rader sequence h[s] = exp(-+2 pi i g^s / R) / M for
// the forward and the inverse transform, the twiddles exp(-2 pi i m / M), the
// index pairs (g^-q mod R, g^q mod R) stored as the bits of a float2, and for
// R = 239 the cos/sin table of its 17-point sub-transforms.
void rader_tables(int R, int g, std::vector<float2> &tab) {
    const int M = R - 1;
    std::vector<int> gp(M), gi(M);
    int ginv = 1;
    for (int e = 0; e < R - 2; ++e) ginv = ginv * g % R;  // g^(R-2) = g^-1
    gp[0] = gi[0] = 1;
    for (int q = 1; q < M; ++q) {
        gp[q] = gp[q - 1] * g % R;
        gi[q] = gi[q - 1] * ginv % R;
    }
    for (int dir = 0; dir < 2; ++dir) {
        const double sgn = dir == 0 ? -1.0 : 1.0;
        for (int k = 0; k < M; ++k) {
            double re = 0.0, im = 0.0;
            for (int s = 0; s < M; ++s) {
                const double a = sgn * 2.0 * M_PI * (double)gp[s] / (double)R;
                const double b = -2.0 * M_PI * (double)((long)s * k % M) / (double)M;
                re += cos(a + b);
                im += sin(a + b);
            }
            tab.push_back(make_float2((float)(re / M), (float)(im / M)));
        }
    }
    for (int m = 0; m < M; ++m) {
        const double a = -2.0 * M_PI * (double)m / (double)M;
        tab.push_back(make_float2((float)cos(a), (float)sin(a)));
    }
    for (int q = 0; q < M; ++q) {
        float2 e;
        memcpy(&e.x, &gi[q], sizeof(int));
        memcpy(&e.y, &gp[q], sizeof(int));
        tab.push_back(e);
    }
    if (R == 239)
        for (int m = 0; m < 17; ++m) {
            const double a = -2.0 * M_PI * (double)m / 17.0;
            tab.push_back(make_float2((float)cos(a), (float)sin(a)));
        }
}
}  // namespace

int mm_fft_plan_get(int n, FftPlan *out) {
    if (n < 1 || n > MM_FFT_MAXN) {
        mm_set_error("FFT length %d outside [1, %d]", n, MM_FFT_MAXN);
        return MM_EINVAL;
    }
    int dev = 0;
    MM_CUDA_TRY(cudaGetDevice(&dev));
    std::lock_guard<std::mutex> lock(g_mu);
    auto it = g_plans.find({dev, n});
    if (it != g_plans.end()) {
        *out = it->second;
        return MM_OK;
    }
    std::vector<int> generic, small;
    factor(n, generic, small);
    FftPlan P = {};
    P.n = n;
    std::vector<float2> tab;
    int Ns = 1;
    // generic (large prime) stages first: at Ns == 1 they need no twiddles
    for (int R : generic) {
        P.rad[P.nst] = R;
        P.ns[P.nst] = Ns;
        P.ptab[P.nst] = (int)tab.size();
        for (int m = 0; m < R; ++m) {
            double a = -2.0 * M_PI * (double)m / (double)R;
            tab.push_back(make_float2((float)cos(a), (float)sin(a)));
        }
        if (R == 113) rader_tables(113, 3, tab);
        if (R == 239) rader_tables(239, 7, tab);
        Ns *= R;
        P.nst++;
    }
    for (int R : small) {
        P.rad[P.nst] = R;
        P.ns[P.nst] = Ns;
        P.ptab[P.nst] = -1;
        if (R >= 11) {
            P.ptab[P.nst] = (int)tab.size();
            for (int m = 0; m < R; ++m) {
                double a = -2.0 * M_PI * (double)m / (double)R;
                tab.push_back(make_float2((float)cos(a), (float)sin(a)));
            }
        }
        Ns *= R;
        P.nst++;
    }
    // stage class (fft.cuh): 0 none, 63 lane primes 41..61, 127 also the lane
    // primes 79, 89 and the Rader stages 113 and 239
    P.lclass = 0;
    for (int i = 0; i < P.nst; ++i) {
        const int R = P.rad[i];
        if (R >= 41 && R <= 61 && P.lclass < 63) P.lclass = 63;
        if (R == 79 || R == 89 || R == 113 || R == 239) P.lclass = 127;
    }
    if (P.nst > MM_FFT_MAXST) {
        mm_set_error("FFT length %d needs too many stages", n);
        return MM_EINVAL;
    }
    std::vector<float2> tw(n);
    for (int m = 0; m < n; ++m) {
        double a = -2.0 * M_PI * (double)m / (double)n;
        tw[m] = make_float2((float)cos(a), (float)sin(a));
    }
    if (tab.empty()) tab.push_back(make_float2(1.f, 0.f));
    P.ntab = (int)tab.size();
    float2 *d_tw = nullptr, *d_tab = nullptr;
    MM_CUDA_TRY(cudaMalloc(&d_tw, sizeof(float2) * n));
    MM_CUDA_TRY(cudaMalloc(&d_tab, sizeof(float2) * tab.size()));
    MM_CUDA_TRY(cudaMemcpy(d_tw, tw.data(), sizeof(float2) * n, cudaMemcpyHostToDevice));
    MM_CUDA_TRY(cudaMemcpy(d_tab, tab.data(), sizeof(float2) * tab.size(), cudaMemcpyHostToDevice));
    P.tw = d_tw;
    P.tab = d_tab;
    g_plans[{dev, n}] = P;
    *out = P;
    return MM_OK;
}
