// memd_synth.cpp -- seeded synthetic inputs and raw .bin I/O (host only).
#include "memd_synth.h"

#include <cmath>
#include <cstdio>
#include <vector>

namespace {

struct Rng {
    uint64_t s[4];
    static uint64_t splitmix(uint64_t& x)
    {
        uint64_t z = (x += 0x9E3779B97F4A7C15ull);
        z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
        z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
        return z ^ (z >> 31);
    }
    explicit Rng(uint64_t seed)
    {
        uint64_t x = seed;
        for (int i = 0; i < 4; ++i) s[i] = splitmix(x);
    }
    static uint64_t rotl(uint64_t x, int k) { return (x << k) | (x >> (64 - k)); }
    uint64_t next()
    {  // xoshiro256**
        const uint64_t r = rotl(s[1] * 5, 7) * 9;
        const uint64_t t = s[1] << 17;
        s[2] ^= s[0];
        s[3] ^= s[1];
        s[1] ^= s[2];
        s[0] ^= s[3];
        s[2] ^= t;
        s[3] = rotl(s[3], 45);
        return r;
    }
    double uniform() { return (double)(next() >> 11) * (1.0 / 9007199254740992.0); }
    double uniform(double a, double b) { return a + (b - a) * uniform(); }
    double normal()
    {
        if (have) {
            have = false;
            return spare;
        }
        double u1 = uniform();
        while (u1 <= 0.0) u1 = uniform();
        const double u2 = uniform();
        const double r = std::sqrt(-2.0 * std::log(u1));
        spare = r * std::sin(2.0 * M_PI * u2);
        have = true;
        return r * std::cos(2.0 * M_PI * u2);
    }
    bool have = false;
    double spare = 0.0;
};

// 1/f noise: white noise through one-pole low-pass sections y = a y + (1-a) x
// whose corners f_j are spaced by a factor 2 from fs/4 down to ~fs/2^17; each
// section has unit gain below its corner, so weights 1/sqrt(f_j) give a summed
// power density close to 1/f across the band.
void pink(Rng& rng, int64_t L, double fs, double* out)
{
    const int nsec = 14;
    double a[nsec], w[nsec], st[nsec];
    double f = fs / 4.0;
    for (int j = 0; j < nsec; ++j) {
        a[j] = std::exp(-2.0 * M_PI * f / fs);
        w[j] = 1.0 / std::sqrt(f);
        st[j] = 0.0;
        f *= 0.5;
    }
    // warm the filters up for three time constants of the slowest section so
    // that the record starts in steady state
    const double f_last = 2.0 * f;
    const double tau = fs / (2.0 * M_PI * f_last);
    const int64_t warm = (int64_t)(3.0 * tau);
    const int64_t nwarm = warm < 200000 ? warm : 200000;
    for (int64_t n = -nwarm; n < L; ++n) {
        const double x = rng.normal();
        double v = 0.0;
        for (int j = 0; j < nsec; ++j) {
            st[j] = a[j] * st[j] + (1.0 - a[j]) * x;
            v += w[j] * st[j];
        }
        if (n >= 0) out[n] = v;
    }
}

}  // namespace

extern "C" int memd_synth_tones(int64_t C, int64_t L, double fs, uint64_t seed, double* out)
{
    if (C < 1 || L < 1 || fs <= 0 || !out) return -1;
    Rng rng(seed);
    const double freqs[3] = {5.0, 20.0, 60.0};
    for (int64_t c = 0; c < C; ++c) {
        double amp[3], ph[3];
        for (int j = 0; j < 3; ++j) {
            amp[j] = rng.uniform(0.5, 1.5);
            ph[j] = rng.uniform(0.0, 2.0 * M_PI);
        }
        for (int64_t n = 0; n < L; ++n) {
            double v = 0.0;
            for (int j = 0; j < 3; ++j) v += amp[j] * std::sin(2.0 * M_PI * freqs[j] * (double)n / fs + ph[j]);
            out[c * L + n] = v + 0.1 * rng.normal();
        }
    }
    return 0;
}

extern "C" int memd_synth_eeg(int64_t C, int64_t L, double fs, uint64_t seed, double* out)
{
    if (C < 1 || L < 1 || fs <= 0 || !out) return -1;
    Rng rng(seed);
    std::vector<double> src((size_t)(C * L));
    for (int64_t c = 0; c < C; ++c) pink(rng, L, fs, &src[(size_t)(c * L)]);
    // normalise each source to unit RMS
    for (int64_t c = 0; c < C; ++c) {
        double ss = 0.0;
        for (int64_t n = 0; n < L; ++n) ss += src[(size_t)(c * L + n)] * src[(size_t)(c * L + n)];
        const double inv = ss > 0 ? 1.0 / std::sqrt(ss / (double)L) : 1.0;
        for (int64_t n = 0; n < L; ++n) src[(size_t)(c * L + n)] *= inv;
    }
    std::vector<double> mix((size_t)(C * C));
    for (auto& m : mix) m = rng.normal() / std::sqrt((double)C);
    for (int64_t i = 0; i < C * L; ++i) out[i] = 0.0;
    for (int64_t c = 0; c < C; ++c)
        for (int64_t j = 0; j < C; ++j) {
            const double m = mix[(size_t)(c * C + j)];
            const double* s = &src[(size_t)(j * L)];
            double* o = out + c * L;
            for (int64_t n = 0; n < L; ++n) o[n] += m * s[n];
        }
    // alpha bursts: Poisson arrivals at 0.2/s, 1-3 s Hann-windowed 10 Hz
    std::vector<double> gain((size_t)C);
    for (auto& g : gain) g = 1.5 * rng.normal();
    double t = 0.0;
    const double dur_total = (double)L / fs;
    while (true) {
        t += -std::log(1.0 - rng.uniform()) / 0.2;
        if (t >= dur_total) break;
        const double d = rng.uniform(1.0, 3.0);
        const double ph = rng.uniform(0.0, 2.0 * M_PI);
        const int64_t n0 = (int64_t)(t * fs);
        const int64_t nd = (int64_t)(d * fs);
        for (int64_t k = 0; k < nd && n0 + k < L; ++k) {
            const double win = 0.5 - 0.5 * std::cos(2.0 * M_PI * (double)k / (double)nd);
            const double v = win * std::sin(2.0 * M_PI * 10.0 * (double)k / fs + ph);
            for (int64_t c = 0; c < C; ++c) out[c * L + n0 + k] += gain[(size_t)c] * v;
        }
    }
    // 0.5 Hz drift and scaling to tens of units
    for (int64_t c = 0; c < C; ++c) {
        const double a = rng.uniform(0.5, 1.5), ph = rng.uniform(0.0, 2.0 * M_PI);
        for (int64_t n = 0; n < L; ++n) {
            double& o = out[c * L + n];
            o = 30.0 * (o + a * std::sin(2.0 * M_PI * 0.5 * (double)n / fs + ph));
        }
    }
    return 0;
}

extern "C" int memd_write_bin(const char* path, const void* data, int64_t count, int32_t elem_bytes)
{
    if (!path || !data || count < 0 || (elem_bytes != 4 && elem_bytes != 8)) return -1;
    FILE* f = std::fopen(path, "wb");
    if (!f) return -2;
    const size_t n = std::fwrite(data, (size_t)elem_bytes, (size_t)count, f);
    std::fclose(f);
    return n == (size_t)count ? 0 : -3;
}

extern "C" int64_t memd_bin_count(const char* path, int32_t elem_bytes)
{
    if (!path || (elem_bytes != 4 && elem_bytes != 8)) return -1;
    FILE* f = std::fopen(path, "rb");
    if (!f) return -2;
    std::fseek(f, 0, SEEK_END);
    const long n = std::ftell(f);
    std::fclose(f);
    return n < 0 ? -3 : (int64_t)n / elem_bytes;
}

extern "C" int memd_read_bin(const char* path, void* data, int64_t count, int32_t elem_bytes)
{
    if (!path || !data || count < 0 || (elem_bytes != 4 && elem_bytes != 8)) return -1;
    FILE* f = std::fopen(path, "rb");
    if (!f) return -2;
    const size_t n = std::fread(data, (size_t)elem_bytes, (size_t)count, f);
    std::fclose(f);
    return n == (size_t)count ? 0 : -3;
}
