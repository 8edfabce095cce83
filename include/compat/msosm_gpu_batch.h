// Drop-in replacement for dedispersion/include/msosm_gpu_batch.h (header-only).
//
// MSOSM_GPU_BATCH with the reference's constructors and methods
// (msosm_gpu_batch.h:13-97) over the engine's C ABI:
//   initialize_uint16(fftpoint, batch, fold)  -> msosm_init(..., MSOSM_IN_U16,
//        fold ? MSOSM_OUT_C64 : MSOSM_OUT_U16)        (msosm_gpu_batch.cpp:12-151)
//   filter_block_uint16(uint16_pair*)         -> msosm_process    (:178-236)
//   get_output(uint16_pair*)                  -> msosm_get_output (:238-245)
//   get_output_pointer()                      -> msosm_device_output
//   synchronize()                             -> msosm_sync
// Differences a caller can see: any batch >= 1 is accepted (the reference needs
// a multiple of 4), the spectra ring starts zeroed, reset_device() and the
// destructor free the handle's memory instead of resetting the whole device,
// and all work is ordered on the legacy default stream.
#pragma once
#include "msosm_prepare.h"
#include "psrdada.h"

constexpr int D2D_REDUCE_COUNT = 1;
constexpr int ITEMS_PER_THREAD = 4;
constexpr int BLOCK_SIZE = 256;

class MSOSM_GPU_BATCH : public Prepare_MSOSM
{
  public:
    MSOSM_GPU_BATCH(float bw = 0, float dm = 0, float f0 = 0) : Prepare_MSOSM(bw, dm, f0) {}
    MSOSM_GPU_BATCH(float bw, float *dm, float f0, int numDMs = 1) : Prepare_MSOSM(bw, dm, f0, numDMs) {}
    ~MSOSM_GPU_BATCH() override { reset_device(); }

    void get_device_info() { cout << msosm_version() << endl; }

    void initialize_uint16(int fftpoint = 0, int batch = 1, bool fold = false)
    {
        this->fold = fold;
        this->batch = batch;
        msosm_compat::check(msosm_create(bw, f0, dm_values, numDMs, &h), nullptr, "MSOSM_GPU_BATCH");
        msosm_compat::check(msosm_init(h, fftpoint, batch, MSOSM_IN_U16, fold ? MSOSM_OUT_C64 : MSOSM_OUT_U16), h,
                            "initialize_uint16");
        int fp = 0;
        msosm_get_dims(h, &M, &M_min, &fp, nullptr, nullptr, &delaycount, &fft_block_size);
        this->fftpoint = fp;
        msosm_get_delaycounts(h, delaycount_values);
        cout << "FFT point: " << fftpoint << endl; // printed unconditionally by the reference
    }
    void filter_block_uint16(uint16_pair *input)
    {
        msosm_compat::check(msosm_process(h, input, nullptr), h, "filter_block_uint16");
        // fold mode returns with the step done, as the reference's synchronous fold-mode
        // branch does (msosm_gpu_batch.cpp:180-202), so `input` may be refilled at once
        if (fold)
            msosm_compat::check(msosm_sync(h, nullptr), h, "filter_block_uint16");
    }
    void get_output(uint16_pair *output) { msosm_compat::check(msosm_get_output(h, output, nullptr), h, "get_output"); }
    void synchronize() { msosm_compat::check(msosm_sync(h, nullptr), h, "synchronize"); }
    void reset_device()
    {
        if (h)
        {
            msosm_sync(h, nullptr);
            msosm_destroy(h);
            h = nullptr;
        }
    }
    Complex *get_output_pointer() { return (Complex *)msosm_device_output(h); }
    msosm_t *handle() { return h; }

  protected:
    bool fold = false;
    int batch = 1;
    int fftpoint = 0;
    int fft_block_size = 0;
    msosm_t *h = nullptr;
};
