/*
 * ORACLE build shim -- a C entry over the reference's own
 * MSOSM_GPU_BATCH::build_segments (msosm_gpu_batch.cpp:262-295), compiled with it
 * into oracle/_ref/libmsosm_ref_seg.so.  Used only by tests/golden/make_golden.py.
 */
#include "msosm_gpu_batch.h"

namespace {
// build_segments is protected: a derived class re-exports it.  The object is never
// destroyed (the processor's destructor resets the device).
struct SegmentProbe : MSOSM_GPU_BATCH
{
    SegmentProbe() : MSOSM_GPU_BATCH(1e6f, 1.0f, 1e9f) {}
    using MSOSM_GPU_BATCH::build_segments;
};
SegmentProbe *probe()
{
    static SegmentProbe *p = new SegmentProbe();
    return p;
}
} // namespace

/* Segments of one per-bin delay map: (start, len, group) triples into out (room for
 * max triples); returns the segment count. */
extern "C" int ref_build_segments(const int *delay, int fft_len, int *out, int max)
{
    const std::vector<Segment> s = probe()->build_segments(delay, fft_len);
    for (size_t i = 0; i < s.size() && (int)i < max; i++)
    {
        out[3 * i] = s[i].start;
        out[3 * i + 1] = s[i].len;
        out[3 * i + 2] = s[i].group;
    }
    return (int)s.size();
}
