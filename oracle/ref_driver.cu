// ref_driver.cu -- command-line driver around the reference MEMD build.
//
// TEST INFRASTRUCTURE ONLY.  oracle/ref_recipe.py writes a lightly patched
// copy of the reference source (memReducedEpochs_dev.cu: the stray text line
// at :1472 commented out, its own main() renamed, and for REF_REAL=double the
// cuBLAS/cuSPARSE S-calls switched to D-calls) into oracle/_ref/, and this
// driver includes that copy.  It runs the reference's own memd<int, REAL>()
// (memReducedEpochs_dev.cu:1074-1368) and GenerateDirectionVector<REAL>()
// (:1029-1072) exactly as the reference's main() does (:1466-1529), but on a
// caller-chosen input file and sizes, so that its IMFs can pin the oracle and
// its run time can be shown beside the GB300 engine.
//
// usage: memd_ref_<f32|f64> in.bin C K num_imfs max_iter out.bin [dirs.bin|-] [repeats]
//   in.bin    C x L raw REAL, channel-major (L = bytes / sizeof(REAL) / C)
//   dirs.bin  K x C raw REAL; "-" or absent: generated by the reference and
//             written to out.bin.dirs
// prints one JSON line: call and loop times.
#include REF_SOURCE

#include <string.h>

static long file_bytes(const char* path)
{
    FILE* f = fopen(path, "rb");
    if (!f) return -1;
    fseek(f, 0, SEEK_END);
    long n = ftell(f);
    fclose(f);
    return n;
}

int main(int argc, char** argv)
{
    typedef REF_REAL real;
    if (argc < 7) {
        fprintf(stderr, "usage: %s in.bin C K num_imfs max_iter out.bin [dirs.bin|-] [repeats]\n", argv[0]);
        return 2;
    }
    const char* in_path = argv[1];
    size_t C = (size_t)atol(argv[2]);
    size_t K = (size_t)atol(argv[3]);
    size_t nimf = (size_t)atol(argv[4]);
    size_t max_iter = (size_t)atol(argv[5]);
    const char* out_path = argv[6];
    const char* dir_path = argc > 7 ? argv[7] : "-";
    int repeats = argc > 8 ? atoi(argv[8]) : 1;
    long nbytes = file_bytes(in_path);
    if (nbytes <= 0 || C == 0 || K == 0 || nimf == 0) {
        fprintf(stderr, "bad input\n");
        return 2;
    }
    size_t L = (size_t)nbytes / sizeof(real) / C;

    real* h_y = (real*)malloc(C * L * sizeof(real));
    FILE* f = fopen(in_path, "rb");
    if (fread(h_y, sizeof(real), C * L, f) != C * L) { fprintf(stderr, "short read\n"); return 2; }
    fclose(f);
    int* h_x = (int*)malloc(L * sizeof(int));
    for (size_t i = 0; i < L; ++i) h_x[i] = (int)i;

    int* d_x = NULL;
    real *d_y = NULL, *d_dir = NULL, *d_imfs = NULL;
    cudaMalloc((void**)&d_x, L * sizeof(int));
    cudaMalloc((void**)&d_y, C * L * sizeof(real));
    cudaMalloc((void**)&d_dir, C * K * sizeof(real));
    cudaMalloc((void**)&d_imfs, nimf * C * L * sizeof(real));
    cudaMemcpy(d_x, h_x, L * sizeof(int), cudaMemcpyHostToDevice);
    cudaMemcpy(d_y, h_y, C * L * sizeof(real), cudaMemcpyHostToDevice);

    real* h_dir = (real*)malloc(C * K * sizeof(real));
    if (strcmp(dir_path, "-") != 0) {
        FILE* fd = fopen(dir_path, "rb");
        if (!fd || fread(h_dir, sizeof(real), C * K, fd) != C * K) { fprintf(stderr, "bad dirs\n"); return 2; }
        fclose(fd);
        cudaMemcpy(d_dir, h_dir, C * K * sizeof(real), cudaMemcpyHostToDevice);
    } else {
        GenerateDirectionVector<real>(C, K, d_dir);
        cudaDeviceSynchronize();
        cudaMemcpy(h_dir, d_dir, C * K * sizeof(real), cudaMemcpyDeviceToHost);
        char dpath[4096];
        snprintf(dpath, sizeof(dpath), "%s.dirs", out_path);
        FILE* fo = fopen(dpath, "wb");
        fwrite(h_dir, sizeof(real), C * K, fo);
        fclose(fo);
    }

    // Guard: the reference hands cusparse<t>gtsv2_nopivot a fixed buffer of
    // 1024*1024 reals and ignores the size query (memReducedEpochs_dev.cu:1144,
    // 1237-1239).  Refuse to run when the library would need more than that
    // for any knot count a direction can have, instead of letting it write past the buffer.
    {
        cusparseHandle_t hs;
        cusparseCreate(&hs);
        real* probe = NULL;
        cudaMalloc((void**)&probe, (L + 8) * C * sizeof(real));
        size_t need_max = 0;
        // A direction has at most L/2 + 2 knots: strict interior maxima
        // (minima) are at least two samples apart, plus both end samples.
        int mmax = (int)((L + 1) / 2 + 2);
        int ms[5] = {3, mmax / 8, mmax / 4, mmax / 2, mmax};
        for (int t = 0; t < 5; ++t) {
            int m = ms[t] < 3 ? 3 : ms[t];
            size_t need = 0;
#if REF_F64
            cusparseDgtsv2_nopivot_bufferSizeExt(hs, m, (int)C, probe, probe, probe, probe, m, &need);
#else
            cusparseSgtsv2_nopivot_bufferSizeExt(hs, m, (int)C, probe, probe, probe, probe, m, &need);
#endif
            if (need > need_max) need_max = need;
        }
        cudaFree(probe);
        cusparseDestroy(hs);
        if (need_max > 1024 * 1024 * sizeof(real)) {
            printf("{\"unavailable\": \"gtsv2 buffer of %zu bytes needed, reference passes %zu\"}\n",
                   need_max, (size_t)(1024 * 1024 * sizeof(real)));
            return 3;
        }
        fprintf(stderr, "gtsv2 buffer need (max over probes): %zu bytes of %zu\n", need_max,
                (size_t)(1024 * 1024 * sizeof(real)));
    }

    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    double best_call_ms = 1e300, best_loop_s = 1e300, sum_call_ms = 0.0;
    for (int r = 0; r < repeats; ++r) {
        cudaDeviceSynchronize();
        cudaEventRecord(e0, 0);
        double loop_s = memd<int, real>(C, L, K, nimf, max_iter, d_x, d_y, d_dir, d_imfs);
        cudaEventRecord(e1, 0);
        cudaEventSynchronize(e1);
        float ms = 0.f;
        cudaEventElapsedTime(&ms, e0, e1);
        if (ms < best_call_ms) best_call_ms = ms;
        if (loop_s < best_loop_s) best_loop_s = loop_s;
        sum_call_ms += ms;
    }
    cudaError_t err = cudaGetLastError();

    real* h_imfs = (real*)malloc(nimf * C * L * sizeof(real));
    cudaMemcpy(h_imfs, d_imfs, nimf * C * L * sizeof(real), cudaMemcpyDeviceToHost);
    FILE* fo = fopen(out_path, "wb");
    fwrite(h_imfs, sizeof(real), nimf * C * L, fo);
    fclose(fo);
    printf("{\"C\": %zu, \"L\": %zu, \"K\": %zu, \"num_imfs\": %zu, \"max_iter\": %zu, \"real_bytes\": %zu, "
           "\"repeats\": %d, \"best_call_ms\": %.4f, \"mean_call_ms\": %.4f, \"best_loop_s\": %.6f, \"cuda_error\": \"%s\"}\n",
           C, L, K, nimf, max_iter, sizeof(real), repeats, best_call_ms, sum_call_ms / repeats, best_loop_s,
           cudaGetErrorString(err));
    return err == cudaSuccess ? 0 : 1;
}
