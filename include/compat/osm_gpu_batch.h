// Drop-in replacement for dedispersion/include/osm_gpu_batch.h and prepare.h
// (header-only): Prepare_OSM (prepare.h:7-40) and OSM_GPU_BATCH
// (osm_gpu_batch.h:7-38) over the engine's C ABI (osm_plan / osm_create).
#pragma once
#include "globals.h"
#include "psrdada.h"

class Prepare_OSM
{
  public:
    Prepare_OSM(float bw = 0, float dm = 0, float f0 = 0) : bw(bw), fs(bw), dm(dm), f0(f0)
    {
        osm_plan(bw, dm, f0, &Nd, nullptr);
    }
    virtual ~Prepare_OSM() { delete[] dedisp_params; }
    void calculate_min_order()
    {
        osm_plan(bw, dm, f0, &Nd, &M_min);
        M = M_min;
    }
    void override_order(unsigned long order) { M = order; }
    void generate_dedisp_params()
    {
        delete[] dedisp_params;
        dedisp_params = new Complex[2 * M];
        msosm_compat::check(msosm_plan_response(bw, f0, dm, (int)M, (float *)dedisp_params), nullptr,
                            "generate_dedisp_params");
    }

  public:
    unsigned long M = 0;
    unsigned long M_min = 0;
    Complex *dedisp_params = nullptr;
    unsigned long Nd = 0;

  protected:
    float bw, fs, dm, f0;
};

class OSM_GPU_BATCH : public Prepare_OSM
{
  public:
    OSM_GPU_BATCH(float bw = 0, float dm = 0, float f0 = 0) : Prepare_OSM(bw, dm, f0) {}
    ~OSM_GPU_BATCH() override
    {
        if (h)
        {
            msosm_sync(h, nullptr);
            msosm_destroy(h);
        }
    }
    void get_device_info() { cout << msosm_version() << endl; }
    void initialize_uint16(unsigned long fftpoint = 0, int batch = 1, bool streaming = false)
    {
        (void)streaming; // work is stream-ordered either way
        this->batch = batch;
        msosm_compat::check(osm_create(bw, dm, f0, &h), nullptr, "OSM_GPU_BATCH");
        msosm_compat::check(msosm_init(h, (int)fftpoint, batch, MSOSM_IN_U16, MSOSM_OUT_C64), h, "initialize_uint16");
        int m = 0, mmin = 0;
        msosm_get_dims(h, &m, &mmin, nullptr, nullptr, nullptr, nullptr, nullptr);
        M = (unsigned long)m;
        M_min = (unsigned long)mmin;
        total_memory = (unsigned long)batch * M * 8 * 5 + 2 * M * 8;
    }
    void filter_block_uint16(uint16_pair *input)
    {
        msosm_compat::check(msosm_process(h, input, nullptr), h, "filter_block_uint16");
    }
    void get_output(Complex *output)
    {
        msosm_compat::check(msosm_get_output(h, output, nullptr), h, "get_output");
        msosm_compat::check(msosm_sync(h, nullptr), h, "get_output");
    }
    Complex *get_output_pointer() { return (Complex *)msosm_device_output(h); }
    msosm_t *handle() { return h; }

  public:
    int batch = 1;
    unsigned long total_memory = 0;

  private:
    msosm_t *h = nullptr;
};
