// Drop-in replacement for the reference's utils/include/globals.h (header-only).
//
// Provides what the reference's executables use from it: the uint16_pair sample
// type (globals.h:22-26), Complex (:29, there cufftComplex), `verbose` (:28),
// `pi` (:30), banner()/line() (:31-32) and the plotting entry points (:34-43).
// Plotting went through embedded matplotlib; here the plot calls write the
// series as text (one value per line) to plot_<n>.txt instead, since the data
// path must not depend on a Python runtime.  No FFTW, cuFFT, NVTX or pybind11
// headers are needed.
#pragma once
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <getopt.h>
#include <iostream>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include <cuda_runtime.h>

#include "../msosm_gb300.h"

using namespace std;

struct __attribute__((packed)) uint16_pair
{
    uint16_t first;
    uint16_t second;
};

struct msosm_complex
{
    float x, y;
};
typedef msosm_complex Complex;

inline bool verbose = false;
constexpr auto pi = M_PI;

inline void line() { cout << string(80, '-') << endl; }
inline void banner() { cout << "MS-OSM coherent dedispersion (GB300 engine, " << msosm_version() << ")" << endl; }

namespace msosm_compat {
inline int &plot_counter()
{
    static int n = 0;
    return n;
}
template <class F>
inline void dump_series(size_t size, F value)
{
    const string name = "plot_" + to_string(plot_counter()++) + ".txt";
    ofstream f(name);
    for (size_t i = 0; i < size; i++)
        f << value(i) << '\n';
}
inline float u16val(uint16_t v) { return v == 0 ? 0.0f : (float)v - 32768.0f; }
} // namespace msosm_compat

inline void plot_init() {}
inline void show() {}
inline void plot_abs(uint16_pair *s, unsigned long size)
{
    msosm_compat::dump_series(size, [&](size_t i) {
        float a = msosm_compat::u16val(s[i].first), b = msosm_compat::u16val(s[i].second);
        return std::sqrt(a * a + b * b);
    });
}
inline void plot_abs(Complex *s, unsigned long size)
{
    msosm_compat::dump_series(size, [&](size_t i) { return std::sqrt(s[i].x * s[i].x + s[i].y * s[i].y); });
}
inline void plot_pol1(uint16_pair *s, unsigned long size)
{
    msosm_compat::dump_series(size, [&](size_t i) { return msosm_compat::u16val(s[i].first); });
}
inline void plot_pol2(uint16_pair *s, unsigned long size)
{
    msosm_compat::dump_series(size, [&](size_t i) { return msosm_compat::u16val(s[i].second); });
}
template <typename T>
inline void plot(T *s, unsigned long size)
{
    msosm_compat::dump_series(size, [&](size_t i) { return s[i]; });
}
inline void plot(vector<double> &v) { msosm_compat::dump_series(v.size(), [&](size_t i) { return v[i]; }); }

// CUDA_CHECK-style failure: print and exit(1), as the reference's processors do
// (gpu/include/gpu_common.cuh:42-62).  The C ABI itself only returns codes.
#ifndef CUDA_CHECK
#define CUDA_CHECK(call)                                                                                    \
    do                                                                                                      \
    {                                                                                                       \
        const cudaError_t msosm_compat_e = (call);                                                          \
        if (msosm_compat_e != cudaSuccess)                                                                  \
        {                                                                                                   \
            cerr << "CUDA error: " << cudaGetErrorString(msosm_compat_e) << " at " << __FILE__ << ":"       \
                 << __LINE__ << endl;                                                                       \
            exit(1);                                                                                        \
        }                                                                                                   \
    } while (0)
#endif
namespace msosm_compat {
inline void check(int rc, msosm_t *h, const char *what)
{
    if (rc != MSOSM_OK)
    {
        cerr << "MS-OSM error in " << what << ": " << msosm_status_string(rc);
        if (h)
            cerr << " (" << msosm_last_error(h) << ")";
        cerr << endl;
        exit(1);
    }
}
} // namespace msosm_compat
