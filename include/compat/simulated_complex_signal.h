// Drop-in replacement for simulated_pulsar/include/simulated_complex_signal.h
// (header-only).
//
// SimulatedComplexSignal with the reference's constructor, generators and public
// members (simulated_complex_signal.h:7-55), generated on the GPU by the engine's
// msosm_sim_* entry points (dispersion through the engine's own overlap-save
// transform, counter-based seeded noise):
//   generate_pulsar_signal_block(dummy, valid)  uint16 only: (dummy + valid) periods
//       of the three-component test pulse times complex Gaussian noise, a new
//       realisation every period, dispersed (simulated_complex_signal.cpp:74-277)
//   generate_pulsar_signal_new(repeat)          the same emission as one continuous
//       dispersed stream, complex (and uint16 when the mode is "uint16") (:279-467)
//   generate_pulsar_signal(repeat, add_noise, SNR, pinned)  two impulses of 32767
//       per period at Np/2 and Np/2 + 2, dispersed, optional AWGN at SNR against the
//       signal power (:469-706); pinned asks for page-locked buffers
// Differences a caller can see: the random sequences differ from the reference's
// mt19937 / default_random_engine draws (same distributions); no simulated_*.bin /
// random_reference.bin cache files are read or written; dispersion smear is limited
// to Nd < 2^23 samples.  As in the reference, the buffers live until the process
// exits (its destructor frees nothing), so they may stay registered with CUDA.
#pragma once
#include "AWGN.h"
#include "globals.h"

#include <cuda_runtime.h>

class SimulatedComplexSignal
{
  public:
    SimulatedComplexSignal(float bw, float dm, float f0, float period, string mode = "complex")
        : data_type(mode), bw(bw), fs(bw), kdm((float)(4.15 * 1e15)), dm(dm), f0(f0), w0((float)(2 * pi * f0)),
          period(period)
    {
        Np = static_cast<unsigned long>(period * fs);
        Nd = static_cast<unsigned long>(floor(kdm * dm * (1 / pow(f0, 2) - 1 / pow(f0 + bw, 2)) / (1 / fs)));
        if (verbose)
        {
            cout << "Test signal parameters:" << endl;
            cout << "Bandwidth: " << bw << "Hz" << endl;
            cout << "Dispersion measure: " << dm << "pc cm^-3" << endl;
            cout << "Start frequency: " << f0 << "Hz" << endl;
            cout << "Pulsar period: " << period << "s" << endl;
            cout << "Period samples: " << Np << endl;
            cout << "Dispersion samples: " << Nd << endl;
            line();
        }
    }

    void generate_pulsar_signal_block(unsigned long dummy_repeat = 0, unsigned long valid_repeat = 1)
    {
        if (data_type != "uint16")
        {
            cout << "Warning: this function is intended for uint16 data type only." << endl;
            return;
        }
        const unsigned long repeat = dummy_repeat + valid_repeat;
        signal_size = repeat * Np;
        range = static_cast<unsigned long>(ceil((double)Nd / (double)Np));
        signal_u16 = (uint16_pair *)alloc(sizeof(uint16_pair) * signal_size, false);
        run(MSOSM_SIM_TEST_PULSE, false, 0.0f, MSOSM_IN_U16, signal_u16);
    }

    void generate_pulsar_signal_new(unsigned long repeat = 1)
    {
        signal_size = repeat * Np;
        range = static_cast<unsigned long>(ceil((double)Nd / (double)Np));
        signal = (fftwf_complex *)alloc(sizeof(fftwf_complex) * signal_size, false);
        run(MSOSM_SIM_TEST_PULSE, false, 0.0f, MSOSM_IN_C64, signal);
        if (data_type == "uint16")
        {
            signal_u16 = (uint16_pair *)alloc(sizeof(uint16_pair) * signal_size, false);
            for (unsigned long i = 0; i < signal_size; i++)
            {
                signal_u16[i].first = static_cast<uint16_t>(signal[i][0] + 32768.0f);
                signal_u16[i].second = static_cast<uint16_t>(signal[i][1] + 32768.0f);
            }
        }
    }

    void generate_pulsar_signal(unsigned long repeat = 1, bool add_noise = false, float SNR = 0, bool pinned = true)
    {
        if (verbose)
            cout << "Generating pulsar signal" << endl;
        signal_size = repeat * Np;
        range = static_cast<unsigned long>(ceil((float)Nd / (float)Np));
        signal = (fftwf_complex *)alloc(sizeof(fftwf_complex) * signal_size, pinned);
        if (data_type == "uint16")
            signal_u16 = (uint16_pair *)alloc(sizeof(uint16_pair) * signal_size, pinned);
        const double power = run(MSOSM_SIM_IMPULSES, add_noise, SNR, MSOSM_IN_C64, signal);
        signal_power = (float)(10 * log10(power));
        if (verbose)
        {
            cout << "Signal measured power: " << signal_power << " dB" << endl;
            line();
        }
        if (data_type == "uint16")
        {
            for (unsigned long i = 0; i < signal_size; i++)
            {
                const float re = signal[i][0], im = signal[i][1];
                if (add_noise)
                {
                    signal_u16[i].first = (re == 0) ? 0 : static_cast<uint16_t>(re + 32768.0f);
                    signal_u16[i].second = (im == 0) ? 0 : static_cast<uint16_t>(im + 32768.0f);
                }
                else
                {
                    signal_u16[i].first = static_cast<uint16_t>(re + 32768.0f);
                    signal_u16[i].second = static_cast<uint16_t>(im + 32768.0f);
                }
            }
        }
    }

    void plot_abs(const fftwf_complex *s, unsigned long size)
    {
        msosm_compat::dump_series(size, [&](size_t i) { return std::sqrt(s[i][0] * s[i][0] + s[i][1] * s[i][1]); });
    }
    void plot_abs(const uint16_pair *s, unsigned long size) { ::plot_abs(const_cast<uint16_pair *>(s), size); }
    ~SimulatedComplexSignal() {}

  public:
    fftwf_complex *signal = nullptr;
    uint16_pair *signal_u16 = nullptr;
    string data_type;
    unsigned long signal_size = 0;
    unsigned long Np = 0;
    unsigned long Nd = 0;
    unsigned long M = 0;
    unsigned long M_min = 0;
    unsigned long range = 0;

  private:
    static void *alloc(size_t bytes, bool pinned)
    {
        void *p = nullptr;
        if (pinned)
        {
            if (cudaMallocHost(&p, bytes) != cudaSuccess)
                p = nullptr;
        }
        else
            p = malloc(bytes);
        if (!p)
        {
            cerr << "SimulatedComplexSignal: allocation of " << bytes << " bytes failed" << endl;
            exit(1);
        }
        return p;
    }
    // signal_size samples of the dispersed stream into `out`; returns the mean power
    double run(int kind, bool noise, float snr_db, int fmt, void *out)
    {
        msosm_sim_t *s = nullptr;
        msosm_compat::check(msosm_sim_create(bw, f0, dm, period, &s), nullptr, "SimulatedComplexSignal");
        auto chk = [&](int rc, const char *what) {
            if (rc != MSOSM_OK)
            {
                cerr << "SimulatedComplexSignal: " << what << ": " << msosm_status_string(rc) << " ("
                     << msosm_sim_last_error(s) << ")" << endl;
                exit(1);
            }
        };
        chk(msosm_sim_set_pulse(s, kind, 0.05f), "set_pulse");
        chk(msosm_sim_set_noise(s, noise ? 1 : 0, snr_db), "set_noise");
        chk(msosm_sim_set_seed(s, 1), "set_seed");
        chk(msosm_sim_generate(s, signal_size, fmt, 1.0f, out, nullptr), "generate");
        double power = 0;
        chk(msosm_sim_info(s, nullptr, nullptr, &power, nullptr), "info");
        msosm_sim_destroy(s);
        return power;
    }

    float bw;
    float fs;
    float kdm;
    float dm;
    float f0;
    float w0;
    float period;
    float signal_power = 0;
};
