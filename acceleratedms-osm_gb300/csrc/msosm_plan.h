// Host-side planning of the MS-OSM engine: smear length, filter order, the
// per-bin block-delay map and the dedispersion response.
//
// Float/double expression types follow the reference's Prepare_MSOSM /
// Prepare_OSM operand by operand (dedispersion/msosm/msosm_prepare.cpp:3-284,
// dedispersion/overlap_save/osm_prepare.cpp:3-140), because they decide the
// integer bin boundaries.  This file is compiled with -ffp-contract=off.
#pragma once
#include <cstdint>
#include <vector>

namespace msosm {

// Nd = floor(kdm*dm * (1/f0^2 - 1/(f0+bw)^2) / (1/fs)), fs = bw (msosm_prepare.cpp:33)
int plan_nd(float bw, float dm, float f0);
unsigned long plan_osm_nd(float bw, float dm, float f0);
// 2^ceil(log2(sqrt(512) * sqrt(Nd))) (msosm_prepare.cpp:48-69)
int plan_min_order(int nd);
// 2*next_pow2((int)Nd) (osm_prepare.cpp:15-28)
unsigned long plan_osm_min_order(unsigned long nd);
// ceil(Nd / (float)M) (msosm_prepare.cpp:217)
int plan_delaycount(int nd, int M);
// segmentation(i) (msosm_prepare.cpp:215-284) -> delay[0..2M).  DM lists with
// delaycount 0 (DM 0) get delay 0 everywhere.  Returns the DM's delaycount.
int plan_segmentation(float bw, float f0, float dm, int nd, int M, uint16_t *delay);
// generate_dedisp_params(i) (msosm_prepare.cpp:107-164), FP64 throughout, rounded
// to complex64 at the end.  Hout: 2M interleaved (re, im) floats.
void plan_response(float bw, float f0, float dm, int M, float *Hout);
// Responses of many DMs on up to `threads` host threads; with derivative set,
// dH/dDM instead (same construction applied to -i (phi/DM) exp(-i phi)).
void plan_responses(float bw, float f0, const float *dms, int n, int M, float *Hout, int threads,
                    bool derivative = false);

// Causal dispersion response for the simulator: the chirp exp(+i phi) sampled at
// fp = next_pow2(nd + 1) bins with the generator's frequency mapping
// (simulated_complex_signal.cpp:347-366), its inverse transform / fp, the
// nd + 1 taps of the physical (negative-time) response moved to indices 0..nd
// (:374-385), zero-padded to F and transformed (:387-389); FP64 throughout,
// rounded to complex64 once.  Hout: F interleaved (re, im) floats; F >= 2 (nd + 1).
void plan_dispersion_response(float bw, float f0, float dm, unsigned long nd, int F, float *Hout);

} // namespace msosm
