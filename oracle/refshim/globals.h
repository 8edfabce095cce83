/*
 * ORACLE build shim -- replaces the reference's utils/include/globals.h for the
 * host-only planning build.  The original also pulls in cufft.h, CUDA runtime,
 * NVTX and pybind11 (plotting), none of which the planning code uses.  This
 * keeps the declarations the planning sources need: the uint16_pair type
 * (globals.h:22-26), `verbose` (:28), `pi` (:30) and line()/banner() (:31-32).
 */
#pragma once
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <iostream>
#include <string>
#include <vector>
#include "fftw3.h"

using namespace std;

struct __attribute__((packed)) uint16_pair
{
    uint16_t first;
    uint16_t second;
};

extern bool verbose;
constexpr auto pi = M_PI;
extern void banner();
extern void line();
