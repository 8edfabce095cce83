/*
 * ORACLE build shim -- a C entry layer over the reference's own planning
 * classes, compiled together with them into oracle/_ref/libmsosm_ref.so.
 * It constructs Prepare_MSOSM / Prepare_OSM exactly as the reference's
 * processors do (MSOSM_GPU_BATCH::initialize_uint16, msosm_gpu_batch.cpp:12-44,
 * 150-189; OSM_GPU_BATCH::initialize_uint16, osm_gpu_batch.cpp:19-45) and copies
 * out Nd, M, delaycount, the per-bin delay map and the response H.
 * Used only by tests/golden/make_golden.py.
 */
#include "msosm_prepare.h"
#include "prepare.h"

bool verbose = false;
void line() {}
void banner() {}

/* Filter order for a DM list (ascending, as the reference requires). */
extern "C" int ref_msosm_order(float bw, float f0, const float *dms, int n, int fftpoint, int *nd_out,
                               int *M_min_out, int *M_out)
{
    float *dm_copy = new float[n];
    std::memcpy(dm_copy, dms, sizeof(float) * n);
    Prepare_MSOSM *p = new Prepare_MSOSM(bw, dm_copy, f0, n);
    p->calculate_min_order();
    int M_min = p->M_min;
    int M = p->M;
    if (fftpoint != 0)
    {
        M = fftpoint / 2;
        if (M < M_min)
            M = M_min;
    }
    for (int i = 0; i < n; i++)
        nd_out[i] = p->Nd_values[i];
    *M_min_out = M_min;
    *M_out = M;
    return 0; /* the reference never frees these objects either */
}

/* delaycount per DM, the processor-wide delaycount, delay maps [n][2M] and
 * responses [n][2M] complex64.  delays_out / H_out may be NULL. */
extern "C" int ref_msosm_tables(float bw, float f0, const float *dms, int n, int M, int *dc_out,
                                int *dc_max_out, int *delays_out, float *H_out)
{
    float *dm_copy = new float[n];
    std::memcpy(dm_copy, dms, sizeof(float) * n);
    Prepare_MSOSM *p = new Prepare_MSOSM(bw, dm_copy, f0, n);
    p->calculate_min_order();
    p->override_order(M);
    const int F = 2 * M;
    for (int i = 0; i < n; i++)
    {
        p->segmentation(i);
        dc_out[i] = p->delaycount_values[i];
        if (delays_out)
        {
            if (dc_out[i] > 0)
                std::memcpy(delays_out + (size_t)i * F, p->delay_points[i], sizeof(int) * F);
            else
                for (int k = 0; k < F; k++)
                    delays_out[(size_t)i * F + k] = -1; /* reference leaves these uninitialised */
        }
        std::free(p->delay_points[i]);
        if (H_out)
        {
            p->generate_dedisp_params(i);
            std::memcpy(H_out + (size_t)i * 2 * F, p->dedisp_params[i], sizeof(float) * 2 * F);
            fftwf_free(p->dedisp_params[i]);
        }
    }
    *dc_max_out = p->delaycount;
    return 0;
}

extern "C" int ref_osm_plan(float bw, float dm, float f0, unsigned long fftpoint, unsigned long *nd_out,
                            unsigned long *M_min_out, unsigned long *M_out, float *H_out)
{
    Prepare_OSM *p = new Prepare_OSM(bw, dm, f0);
    p->calculate_min_order();
    unsigned long M_min = p->M_min;
    unsigned long M = p->M;
    if (fftpoint != 0)
    {
        M = fftpoint / 2;
        if (M < M_min)
            M = M_min;
    }
    p->override_order(M);
    *nd_out = p->Nd;
    *M_min_out = M_min;
    *M_out = M;
    if (H_out)
    {
        p->generate_dedisp_params();
        std::memcpy(H_out, p->dedisp_params, sizeof(float) * 2 * 2 * M);
        fftwf_free(p->dedisp_params);
    }
    return 0;
}
