// sample_synthetic_signal.cpp -- the driver the reference's README builds
// beside memReducedEpochs_dev.cu (README.md:14; the file is not in the
// reference), written against the drop-in template entry points: it follows
// the reference's main() (memReducedEpochs_dev.cu:1466-1529) step by step on a
// synthetic record instead of EEGsample_32CH_30504.bin.
//
// Signal: 8 channels x 2000 samples at fs = 1 kHz, each channel tones at 5, 20
// and 60 Hz with amplitudes U[0.5, 1.5] and phases U[0, 2 pi) plus
// N(0, 0.1^2) noise, seed 0; 64 directions, 9 IMF slots, 10 sifts per IMF.
//
//   sample_synthetic_signal [out.bin] [f64|f32]
// writes the IMFs (num_IMFs x C x L, raw little-endian) like mode_matrix.bin.
#include <cuda_runtime.h>

#include <cstdio>
#include <cstring>
#include <vector>

#include "memd_reference.hpp"
#include "memd_synth.h"

template <typename real>
static int run(const char* out_path)
{
    size_t SignalDim = 8;
    size_t SignalLength = 2000;
    size_t NumDirVector = 64;
    size_t num_IMFs = 9;
    size_t max_iter = 10;

    std::vector<double> y64(SignalDim * SignalLength);
    memd_synth_tones((int64_t)SignalDim, (int64_t)SignalLength, 1000.0, 0, y64.data());
    std::vector<real> h_y(y64.begin(), y64.end());
    std::vector<int> h_x(SignalLength);
    for (size_t i = 0; i < SignalLength; ++i) h_x[i] = (int)i;

    int* d_x = nullptr;
    real *d_y = nullptr, *d_dir = nullptr, *d_IMFs = nullptr;
    cudaMalloc((void**)&d_x, SignalLength * sizeof(int));
    cudaMalloc((void**)&d_y, SignalDim * SignalLength * sizeof(real));
    cudaMalloc((void**)&d_dir, SignalDim * NumDirVector * sizeof(real));
    cudaMalloc((void**)&d_IMFs, num_IMFs * SignalDim * SignalLength * sizeof(real));
    cudaMemcpy(d_x, h_x.data(), SignalLength * sizeof(int), cudaMemcpyHostToDevice);
    cudaMemcpy(d_y, h_y.data(), SignalDim * SignalLength * sizeof(real), cudaMemcpyHostToDevice);

    GenerateDirectionVector<real>(SignalDim, NumDirVector, d_dir);
    double t = memd<int, real>(SignalDim, SignalLength, NumDirVector, num_IMFs, max_iter, d_x, d_y, d_dir, d_IMFs);

    std::vector<real> IMFs(num_IMFs * SignalDim * SignalLength);
    cudaMemcpy(IMFs.data(), d_IMFs, IMFs.size() * sizeof(real), cudaMemcpyDeviceToHost);
    const int rc = memd_write_bin(out_path, IMFs.data(), (int64_t)IMFs.size(), (int32_t)sizeof(real));
    std::printf("memd: %zu channels x %zu samples, %zu directions, %zu IMF slots: %.3f ms -> %s\n", SignalDim,
                SignalLength, NumDirVector, num_IMFs, t * 1e3, out_path);
    cudaFree(d_x);
    cudaFree(d_y);
    cudaFree(d_dir);
    cudaFree(d_IMFs);
    return (t < 0 || rc != 0) ? 1 : 0;
}

int main(int argc, char** argv)
{
    const char* out = argc > 1 ? argv[1] : "./mode_matrix.bin";
    const bool f32 = argc > 2 && std::strcmp(argv[2], "f32") == 0;
    return f32 ? run<float>(out) : run<double>(out);
}
