// Drop-in replacement for folding/include/fold_gpu.h (header-only): Fold_GPU
// (fold_gpu.h:10-43) over the engine's fold object.  calculate_intensity records
// the processors' device outputs; fold_data_phase computes the intensity
// (|a|^2 for one pol, sqrt(|a|^2+|b|^2) for two) and folds it in one pass, so
// no intensity buffer exists.  get_folded_data/write_to_file behave as in the
// reference (fold_gpu.cpp:56-68).
#pragma once
#include "globals.h"
#include "msosm_gpu_batch.h"
#include "osm_gpu_batch.h"

class Fold_GPU
{
  public:
    Fold_GPU(float period, float fs, unsigned long size, string outfileName = "fold.txt",
             unsigned long time_bin = (unsigned long)-1)
        : size(size)
    {
        period_samples_float = period * fs;
        period_samples = (unsigned long)period_samples_float;
        const unsigned long K = (time_bin == (unsigned long)-1) ? 0 : time_bin;
        msosm_compat::check(msosm_fold_create(period, fs, size, K, 1, &f), nullptr, "Fold_GPU");
        msosm_fold_dims(f, &this->time_bin, nullptr, nullptr);
        folded_data = new float[this->time_bin]();
        outfile.open(outfileName);
    }
    ~Fold_GPU()
    {
        outfile.close();
        msosm_fold_destroy(f);
        delete[] folded_data;
    }
    template <typename T>
    void calculate_intensity(T *pol1, T *pol2)
    {
        a = pol1->get_output_pointer();
        b = pol2->get_output_pointer();
    }
    template <typename T>
    void calculate_intensity(T *pol1)
    {
        a = pol1->get_output_pointer();
        b = nullptr;
    }
    void fold_data_phase() { msosm_compat::check(msosm_fold_accumulate(f, a, b, nullptr), nullptr, "fold_data_phase"); }
    void get_folded_data()
    {
        msosm_compat::check(msosm_fold_read(f, folded_data, nullptr, nullptr, nullptr), nullptr, "get_folded_data");
    }
    void write_to_file()
    {
        for (unsigned long i = 0; i < time_bin; i++)
            outfile << folded_data[i] << endl;
    }
    // the engine's fold handle, for callers that mix the class with the C ABI
    msosm_fold_t *handle() { return f; }

  public:
    float *folded_data = nullptr;
    unsigned long time_bin = 0;
    unsigned long period_samples = 0;

  private:
    unsigned long size;
    float period_samples_float;
    msosm_fold_t *f = nullptr;
    const void *a = nullptr, *b = nullptr;
    ofstream outfile;
};
