// Drop-in replacement for dedispersion/include/msosm_prepare.h (header-only).
//
// Prepare_MSOSM (msosm_prepare.h:9-60) with the same public members and methods;
// the arithmetic runs in the engine's host planning code through the C ABI
// (msosm_plan_*), which reproduces the reference's integer results bit for bit.
// dedisp_params holds complex64 responses (the reference's fftwf_complex**).
#pragma once
#include "globals.h"

constexpr int MIN_SEGMENT_POINTS = 1024;

class Prepare_MSOSM
{
  public:
    Prepare_MSOSM(float bw = 0, float dm = 0, float f0 = 0) : numDMs(1), bw(bw), fs(bw), f0(f0)
    {
        own_dm.assign(1, dm);
        dm_values = own_dm.data();
        setup();
    }
    Prepare_MSOSM(float bw, float *dm, float f0, int numDMs = 1) : numDMs(numDMs), bw(bw), fs(bw), f0(f0)
    {
        dm_values = dm; // borrowed for the object's lifetime, as in the reference
        setup();
    }
    virtual ~Prepare_MSOSM()
    {
        for (int i = 0; i < numDMs; i++)
        {
            delete[] delay_points[i];
            delete[] dedisp_params[i];
        }
        delete[] delay_points;
        delete[] dedisp_params;
        delete[] delaycount_values;
        delete[] Nd_values;
        delete[] M_values;
    }
    void calculate_min_order()
    {
        delete[] M_values;
        M_values = new int[numDMs];
        for (int i = 0; i < numDMs; i++)
            msosm_plan_min_order(&Nd_values[i], 1, &M_values[i]);
        M = *std::max_element(M_values, M_values + numDMs);
        M_min = M;
    }
    void override_order(int order) { M = order; }
    void generate_dedisp_params(int i = 0)
    {
        delete[] dedisp_params[i];
        dedisp_params[i] = new Complex[2 * (size_t)M];
        msosm_compat::check(msosm_plan_response(bw, f0, dm_values[i], M, (float *)dedisp_params[i]), nullptr,
                            "generate_dedisp_params");
    }
    void segmentation(int i = 0)
    {
        delete[] delay_points[i];
        delay_points[i] = new int[2 * (size_t)M];
        msosm_compat::check(
            msosm_plan_segmentation(bw, f0, dm_values[i], Nd_values[i], M, delay_points[i], &delaycount_values[i]),
            nullptr, "segmentation");
        delaycount = std::max(delaycount, delaycount_values[i]);
    }

  public:
    int numDMs;
    int M = 0;
    int M_min = 0;
    int *M_values = nullptr;
    int delaycount = 0;
    int *delaycount_values = nullptr;
    Complex **dedisp_params = nullptr;
    int **delay_points = nullptr;
    int *Nd_values = nullptr;
    int start_Nd = 0;
    int end_Nd = 0;

  protected:
    float bw, fs, kdm = (float)(4.15 * 1e15);
    float *dm_values = nullptr;
    float f0, w0 = 0;
    std::vector<float> own_dm;

  private:
    void setup()
    {
        w0 = (float)(2 * pi * f0);
        Nd_values = new int[numDMs];
        if (numDMs > 0)
            msosm_plan_nd(bw, f0, dm_values, numDMs, Nd_values);
        start_Nd = numDMs > 0 ? Nd_values[0] : 0;
        end_Nd = numDMs > 0 ? Nd_values[numDMs - 1] : 0;
        dedisp_params = new Complex *[numDMs]();
        delay_points = new int *[numDMs]();
        delaycount_values = new int[numDMs]();
        if (verbose)
            for (int i = 0; i < numDMs; i++)
                cout << "Dispersion smearing points for DM " << dm_values[i] << ": " << Nd_values[i] << endl;
    }
};
