// Drop-in replacement for simulated_pulsar/include/AWGN.h (header-only).
//
// AWGN with the reference's constructors and generateNoiseSamples()/deallocate()
// (AWGN.h:8-17, AWGN.cpp:3-64), generated on the GPU by msosm_awgn.  As in the
// reference: the SNR constructor gives quadratures of standard deviation
// sqrt(10^(-SNR/10)) / sqrt(2); the (mean, variance, n) constructor passes
// `variance` to the normal distribution as its standard deviation, as
// std::normal_distribution(mean, variance) does there; every object draws the
// same sequence (the reference default-constructs its engine on each call; here a
// fixed seed of the counter-based generator).  Samples are complex single-precision
// pairs in a host buffer that deallocate() frees.  No FFTW header is needed.
#pragma once
#include <cmath>
#include <cstdlib>
#include <iostream>
#include <random>
#include <vector>

#include "../msosm_gb300.h"

using namespace std;

#ifndef MSOSM_COMPAT_FFTWF_COMPLEX
#define MSOSM_COMPAT_FFTWF_COMPLEX
typedef float fftwf_complex[2]; // FFTW's single-precision complex layout
#endif

class AWGN
{
  public:
    AWGN() : mean(0.0f), variance(1.0f), numberOfSamples(100), sigma(1.0f), isSNRMode(false) {}
    AWGN(float mean, float variance, unsigned long numberOfSamples)
        : mean(mean), variance(variance), numberOfSamples(numberOfSamples), sigma(1.0f), isSNRMode(false)
    {
    }
    AWGN(float SNR, unsigned long numberOfSamples)
        : mean(0.0f), variance(1.0f), numberOfSamples(numberOfSamples), sigma((float)sqrt(pow(10, (-SNR / 10)))),
          isSNRMode(true)
    {
    }

    fftwf_complex *generateNoiseSamples()
    {
        samples = (fftwf_complex *)malloc(numberOfSamples * sizeof(fftwf_complex));
        if (!samples)
        {
            cerr << "AWGN: allocation of " << numberOfSamples << " samples failed" << endl;
            exit(1);
        }
        const float m = isSNRMode ? 0.0f : mean;
        const float sd = isSNRMode ? sigma / (float)sqrt(2.0) : variance;
        const int rc = msosm_awgn(kSeed, 0, numberOfSamples, m, sd, (float *)samples, nullptr);
        if (rc != MSOSM_OK)
        {
            cerr << "AWGN: msosm_awgn failed: " << msosm_status_string(rc) << endl;
            exit(1);
        }
        return samples;
    }
    void deallocate()
    {
        free(samples);
        samples = nullptr;
    }

  private:
    static constexpr unsigned long long kSeed = 5489; // one fixed sequence, as the default-seeded engine
    float mean;
    float variance;
    unsigned long numberOfSamples;
    float sigma;
    bool isSNRMode;
    fftwf_complex *samples = nullptr;
};
