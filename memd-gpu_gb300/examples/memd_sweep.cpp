// memd_sweep.cpp -- the reference's benchmark sweep (runBenchmark,
// memReducedEpochs_dev.cu:1370-1464) over the C ABI: for every channel count,
// direction count and record length, decompose a record with num_IMFs slots x
// max_iter sifts and print "Channel, Length, DirVec, Time" (Time: seconds per
// decomposition, as memd() returns, REF:1336-1337 and 1449).
//
//   memd_sweep [--channels 32,64,128] [--directions 64,128,256]
//              [--lengths 2049:241665:2048] [--imfs 8] [--iter 10]
//              [--precision f64|f32|mixed] [--repeats R] [--seed S]
//
// The reference reads InputData_{C}CH_244032.bin (not shipped with it); the
// sweep uses the seeded EEG-shaped generator (memd_synth.h) instead, the
// first L samples of one record of 244,032 samples per channel count, as the
// reference takes the first L samples of its file.  Each point runs once to
// build the plan and graph, then R timed repeats (the minimum is printed).
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "memd_gb300.h"
#include "memd_synth.h"

static std::vector<int64_t> parse_list(const char* s)
{
    std::vector<int64_t> v;
    std::string t(s);
    size_t pos = 0;
    while (pos <= t.size()) {
        const size_t q = t.find(',', pos);
        const std::string item = t.substr(pos, q == std::string::npos ? std::string::npos : q - pos);
        if (!item.empty()) v.push_back(std::atoll(item.c_str()));
        if (q == std::string::npos) break;
        pos = q + 1;
    }
    return v;
}

static void usage()
{
    std::fprintf(stderr,
                 "usage: memd_sweep [--channels 32,64,128] [--directions 64,128,256] [--lengths 2049:241665:2048]\n"
                 "                  [--imfs 8] [--iter 10] [--precision f64|f32|mixed] [--repeats R] [--seed S]\n");
}

int main(int argc, char** argv)
{
    std::vector<int64_t> chans = {32, 64, 128}, dirs = {64, 128, 256};
    int64_t l0 = 2049, l1 = 241665, ls = 2048, nimf = 8, iter = 10, reps = 1;
    uint64_t seed = 0;
    std::string prec_s = "f32";
    for (int i = 1; i < argc; ++i) {
        const std::string a = argv[i];
        auto next = [&](void) -> const char* {
            if (i + 1 >= argc) {
                usage();
                std::exit(2);
            }
            return argv[++i];
        };
        if (a == "--channels") chans = parse_list(next());
        else if (a == "--directions") dirs = parse_list(next());
        else if (a == "--lengths") {
            const char* v = next();
            if (std::sscanf(v, "%lld:%lld:%lld", (long long*)&l0, (long long*)&l1, (long long*)&ls) != 3) {
                usage();
                return 2;
            }
        } else if (a == "--imfs") nimf = std::atoll(next());
        else if (a == "--iter") iter = std::atoll(next());
        else if (a == "--precision") prec_s = next();
        else if (a == "--repeats") reps = std::max<int64_t>(1, std::atoll(next()));
        else if (a == "--seed") seed = std::strtoull(next(), nullptr, 10);
        else if (a == "--help" || a == "-h") {
            usage();
            return 0;
        } else {
            usage();
            return 2;
        }
    }
    int prec = MEMD_PREC_F32;
    if (prec_s == "f64") prec = MEMD_PREC_F64;
    else if (prec_s == "mixed") prec = MEMD_PREC_MIXED;
    else if (prec_s != "f32") {
        usage();
        return 2;
    }
    if (chans.empty() || dirs.empty() || ls < 1 || l0 < 4 || l1 < l0) {
        usage();
        return 2;
    }
    const size_t es = prec == MEMD_PREC_F64 ? 8 : 4;
    const int64_t Lfile = 244032;  // samples per channel of the reference's input files
    std::printf("Channel, Length, DirVec, Time\n");
    for (int64_t C : chans) {
        std::vector<double> rec((size_t)(C * Lfile));
        if (memd_synth_eeg(C, Lfile, 256.0, seed + (uint64_t)C, rec.data()) != MEMD_OK) {
            std::fprintf(stderr, "memd_sweep: synth: %s\n", memd_last_error());
            return 1;
        }
        for (int64_t K : dirs) {
            void* d_dir = nullptr;
            if (cudaMalloc(&d_dir, es * (size_t)(K * C)) != cudaSuccess) return 1;
            memd_status st = es == 8 ? memd_directions_f64(C, K, nullptr, (double*)d_dir, nullptr)
                                     : memd_directions_f32(C, K, nullptr, (float*)d_dir, nullptr);
            if (st != MEMD_OK) {
                std::fprintf(stderr, "memd_sweep: directions: %s\n", memd_last_error());
                return 1;
            }
            for (int64_t L = l0; L <= l1 && L <= Lfile; L += ls) {
                // first L samples of every channel, channel-major
                std::vector<char> host((size_t)(C * L) * es);
                for (int64_t c = 0; c < C; ++c)
                    for (int64_t n = 0; n < L; ++n) {
                        const double v = rec[(size_t)(c * Lfile + n)];
                        if (es == 8) ((double*)host.data())[c * L + n] = v;
                        else ((float*)host.data())[c * L + n] = (float)v;
                    }
                void *d_y = nullptr, *d_imf = nullptr;
                if (cudaMalloc(&d_y, host.size()) != cudaSuccess ||
                    cudaMalloc(&d_imf, host.size() * (size_t)nimf) != cudaSuccess) {
                    std::fprintf(stderr, "memd_sweep: out of device memory at C=%lld L=%lld\n", (long long)C,
                                 (long long)L);
                    return 1;
                }
                cudaMemcpy(d_y, host.data(), host.size(), cudaMemcpyHostToDevice);
                memd_config cfg;
                memd_default_config(&cfg);
                cfg.channels = C;
                cfg.length = L;
                cfg.directions = K;
                cfg.num_imfs = nimf;
                cfg.max_iter = iter;
                cfg.precision = prec;
                memd_plan* plan = nullptr;
                if (memd_plan_create(&cfg, &plan) != MEMD_OK) {
                    std::fprintf(stderr, "memd_sweep: plan: %s\n", memd_last_error());
                    return 1;
                }
                double best = 1e30;
                for (int64_t r = 0; r <= reps; ++r) {  // run 0 builds the graph
                    memd_stats stats;
                    st = es == 8 ? memd_run_f64(plan, nullptr, (const double*)d_y, (const double*)d_dir,
                                                (double*)d_imf, nullptr, &stats)
                                 : memd_run_f32(plan, nullptr, (const float*)d_y, (const float*)d_dir,
                                                (float*)d_imf, nullptr, &stats);
                    if (st != MEMD_OK) {
                        std::fprintf(stderr, "memd_sweep: run: %s\n", memd_last_error());
                        return 1;
                    }
                    if (r > 0) best = std::min(best, stats.elapsed_ms * 1e-3);
                }
                std::printf("%lld, %lld, %lld, %.6f\n", (long long)C, (long long)L, (long long)K, best);
                std::fflush(stdout);
                memd_plan_destroy(plan);
                cudaFree(d_y);
                cudaFree(d_imf);
            }
            cudaFree(d_dir);
        }
    }
    return 0;
}
