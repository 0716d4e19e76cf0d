// memd_cli.cpp -- command-line decomposition of raw .bin records in the
// reference's file format (memReducedEpochs_dev.cu:896-932, 1484-1527: raw
// little-endian values, channel-major, no header; IMFs written the same way).
//
//   memd_cli --in x.bin --channels C [--f64] [--directions K] [--imfs N]
//            [--iter M] [--precision f64|f32|mixed] [--stop [--sd v --sd2 v --tol v]]
//            [--mex-primes] [--full-window] [--spline natural|nak]
//            [--boundary reference|mirror] --out mode_matrix.bin
//   memd_cli --synthetic eeg|tones --channels C --length L [--seed S] ...
//
// Input values are float32 unless --f64; the IMFs are written in the input's
// type.  --mex-primes builds the direction set with the MEX convention (the
// first C primes) instead of the standalone table.  --spline nak selects
// not-a-knot envelope splines, --boundary mirror the mirrored end extrema
// (both off by default: the reference's natural splines and end clamp).
#include <cuda_runtime.h>

#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "memd_gb300.h"
#include "memd_synth.h"

static void usage()
{
    std::fprintf(stderr,
                 "usage: memd_cli (--in FILE | --synthetic eeg|tones --length L [--seed S]) --channels C\n"
                 "                [--f64] [--directions K] [--imfs N] [--iter M] [--precision f64|f32|mixed]\n"
                 "                [--stop [--sd v] [--sd2 v] [--tol v]] [--mex-primes] [--full-window]\n"
                 "                [--spline natural|nak] [--boundary reference|mirror] --out FILE\n");
}

int main(int argc, char** argv)
{
    std::string in, out, synth, prec_s, spline_s, bound_s;
    int64_t C = 0, L = 0, K = 64, nimf = 9, iter = 10;
    uint64_t seed = 0;
    bool f64 = false, stop = false, mex = false, full = false;
    double sd = 0.075, sd2 = 0.75, tol = 0.075;
    for (int i = 1; i < argc; ++i) {
        std::string a = argv[i];
        auto next = [&](void) -> const char* {
            if (i + 1 >= argc) {
                usage();
                std::exit(2);
            }
            return argv[++i];
        };
        if (a == "--in") in = next();
        else if (a == "--out") out = next();
        else if (a == "--synthetic") synth = next();
        else if (a == "--channels") C = std::atoll(next());
        else if (a == "--length") L = std::atoll(next());
        else if (a == "--seed") seed = std::strtoull(next(), nullptr, 10);
        else if (a == "--directions") K = std::atoll(next());
        else if (a == "--imfs") nimf = std::atoll(next());
        else if (a == "--iter") iter = std::atoll(next());
        else if (a == "--precision") prec_s = next();
        else if (a == "--f64") f64 = true;
        else if (a == "--stop") stop = true;
        else if (a == "--sd") sd = std::atof(next());
        else if (a == "--sd2") sd2 = std::atof(next());
        else if (a == "--tol") tol = std::atof(next());
        else if (a == "--mex-primes") mex = true;
        else if (a == "--full-window") full = true;
        else if (a == "--spline") spline_s = next();
        else if (a == "--boundary") bound_s = next();
        else if (a == "--help" || a == "-h") {
            usage();
            return 0;
        } else {
            std::fprintf(stderr, "unknown argument %s\n", a.c_str());
            usage();
            return 2;
        }
    }
    if (C < 1 || out.empty() || (in.empty() && synth.empty())) {
        usage();
        return 2;
    }
    const int eb = f64 ? 8 : 4;
    std::vector<double> y;
    if (!in.empty()) {
        const int64_t n = memd_bin_count(in.c_str(), eb);
        if (n <= 0 || n % C) {
            std::fprintf(stderr, "cannot read %s as %lld channels\n", in.c_str(), (long long)C);
            return 1;
        }
        L = n / C;
        y.resize((size_t)n);
        if (f64) {
            if (memd_read_bin(in.c_str(), y.data(), n, 8)) return 1;
        } else {
            std::vector<float> t((size_t)n);
            if (memd_read_bin(in.c_str(), t.data(), n, 4)) return 1;
            for (int64_t i = 0; i < n; ++i) y[(size_t)i] = t[(size_t)i];
        }
    } else {
        if (L < 4) {
            std::fprintf(stderr, "--length >= 4 needed\n");
            return 2;
        }
        y.resize((size_t)(C * L));
        const int rc = synth == "tones" ? memd_synth_tones(C, L, 1000.0, seed, y.data())
                                        : memd_synth_eeg(C, L, 256.0, seed, y.data());
        if (rc) return 1;
    }
    memd_config cfg;
    memd_default_config(&cfg);
    cfg.channels = C;
    cfg.length = L;
    cfg.directions = K;
    cfg.num_imfs = nimf;
    cfg.max_iter = iter;
    cfg.precision = f64 ? MEMD_PREC_F64 : MEMD_PREC_F32;
    if (prec_s == "f64") cfg.precision = MEMD_PREC_F64;
    else if (prec_s == "f32") cfg.precision = MEMD_PREC_F32;
    else if (prec_s == "mixed") cfg.precision = MEMD_PREC_MIXED;
    if (stop) {
        cfg.stop_mode = MEMD_STOP_CRITERION;
        cfg.stop_sd = sd;
        cfg.stop_sd2 = sd2;
        cfg.stop_tol = tol;
    }
    if (full) cfg.ref_window = 0;
    if (!spline_s.empty() && spline_s != "natural" && spline_s != "nak") {
        std::fprintf(stderr, "--spline natural|nak\n");
        return 2;
    }
    if (!bound_s.empty() && bound_s != "reference" && bound_s != "mirror") {
        std::fprintf(stderr, "--boundary reference|mirror\n");
        return 2;
    }
    if (spline_s == "nak") cfg.spline_end = MEMD_SPLINE_NOT_A_KNOT;
    if (bound_s == "mirror") cfg.boundary = MEMD_BOUNDARY_MIRROR;
    memd_plan* plan = nullptr;
    if (memd_plan_create(&cfg, &plan) != MEMD_OK) {
        std::fprintf(stderr, "plan: %s\n", memd_last_error());
        return 1;
    }
    std::vector<int32_t> primes;
    if (mex) {
        int cand = 2;
        while ((int64_t)primes.size() < C) {
            bool comp = false;
            for (int d = 2; d * d <= cand; ++d)
                if (cand % d == 0) { comp = true; break; }
            if (!comp) primes.push_back(cand);
            ++cand;
        }
    }
    const size_t CL = (size_t)(C * L), NO = (size_t)nimf * CL;
    memd_stats st;
    memd_status rc;
    std::vector<double> imf64;
    std::vector<float> imf32;
    if (cfg.precision == MEMD_PREC_F64) {
        double *dy, *dd, *dout;
        cudaMalloc((void**)&dy, CL * 8);
        cudaMalloc((void**)&dd, (size_t)(K * C) * 8);
        cudaMalloc((void**)&dout, NO * 8);
        cudaMemcpy(dy, y.data(), CL * 8, cudaMemcpyHostToDevice);
        rc = memd_directions_f64(C, K, mex ? primes.data() : nullptr, dd, nullptr);
        if (rc == MEMD_OK) rc = memd_run_f64(plan, nullptr, dy, dd, dout, nullptr, &st);
        imf64.resize(NO);
        cudaMemcpy(imf64.data(), dout, NO * 8, cudaMemcpyDeviceToHost);
        cudaFree(dy);
        cudaFree(dd);
        cudaFree(dout);
    } else {
        std::vector<float> y32(y.begin(), y.end());
        float *dy, *dd, *dout;
        cudaMalloc((void**)&dy, CL * 4);
        cudaMalloc((void**)&dd, (size_t)(K * C) * 4);
        cudaMalloc((void**)&dout, NO * 4);
        cudaMemcpy(dy, y32.data(), CL * 4, cudaMemcpyHostToDevice);
        rc = memd_directions_f32(C, K, mex ? primes.data() : nullptr, dd, nullptr);
        if (rc == MEMD_OK) rc = memd_run_f32(plan, nullptr, dy, dd, dout, nullptr, &st);
        imf32.resize(NO);
        cudaMemcpy(imf32.data(), dout, NO * 4, cudaMemcpyDeviceToHost);
        cudaFree(dy);
        cudaFree(dd);
        cudaFree(dout);
    }
    memd_plan_destroy(plan);
    if (rc != MEMD_OK) {
        std::fprintf(stderr, "run: %s\n", memd_last_error());
        return 1;
    }
    int wrc;
    if (f64) {
        if (imf64.empty()) imf64.assign(imf32.begin(), imf32.end());
        wrc = memd_write_bin(out.c_str(), imf64.data(), (int64_t)NO, 8);
    } else {
        if (imf32.empty()) imf32.assign(imf64.begin(), imf64.end());
        wrc = memd_write_bin(out.c_str(), imf32.data(), (int64_t)NO, 4);
    }
    std::printf("{\"channels\": %lld, \"length\": %lld, \"directions\": %lld, \"n_imfs\": %d, \"elapsed_ms\": %.4f, "
                "\"flags\": %d, \"out\": \"%s\"}\n",
                (long long)C, (long long)L, (long long)K, st.n_imfs, st.elapsed_ms, st.flags, out.c_str());
    return wrc ? 1 : 0;
}
