/*
 * memd_synth.h -- seeded synthetic multichannel signals (host, C ABI).
 *
 * The reference ships one real EEG record and reads benchmark inputs
 * (InputData_{32,64,128}CH_244032.bin, memReducedEpochs_dev.cu:1377-1379) that
 * it does not ship; these generators stand in for them.  Output layout is the
 * reference's: C x L, channel-major, host memory.  Deterministic for a seed
 * (xoshiro256** seeded by splitmix64, Box-Muller normals).
 */
#ifndef MEMD_SYNTH_H
#define MEMD_SYNTH_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Tones at 5, 20 and 60 Hz with per-channel amplitudes U[0.5, 1.5] and
 * phases U[0, 2 pi), plus N(0, 0.1^2) noise. */
int memd_synth_tones(int64_t channels, int64_t length, double fs, uint64_t seed, double* out);

/* EEG-shaped: C independent 1/f sources (sum of one-pole sections with
 * geometrically spaced corners) mixed by a seeded C x C Gaussian matrix, plus
 * 10 Hz Hann-windowed alpha bursts (1-3 s long, Poisson rate 0.2/s, per-channel
 * gains) and a 0.5 Hz drift; scaled to tens of units like the reference's
 * EEG sample. */
int memd_synth_eeg(int64_t channels, int64_t length, double fs, uint64_t seed, double* out);

/* Writes / reads raw little-endian arrays in the reference's .bin format (no
 * header; memReducedEpochs_dev.cu:896-932).  elem_bytes 4 (float32) or 8. */
int memd_write_bin(const char* path, const void* data, int64_t count, int32_t elem_bytes);
int64_t memd_bin_count(const char* path, int32_t elem_bytes);
int memd_read_bin(const char* path, void* data, int64_t count, int32_t elem_bytes);

#ifdef __cplusplus
}
#endif

#endif /* MEMD_SYNTH_H */
