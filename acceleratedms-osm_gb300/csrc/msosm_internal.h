// Entry points the library's own components share (not part of the public C ABI).
#pragma once
#include "msosm_gb300.h"

// An overlap-save handle of one filter with a caller-chosen order M (a power of two,
// F = 2M): every bin has block delay 0, as for osm_create, but M is not derived
// from a DM.  msosm_init(h, 2*M, ...) and msosm_set_response then make it apply any
// F-bin response, e.g. the simulator's dispersion.
int msosm_filter_create(float bw, float f0, int M, msosm_t **out);
