// Persistent inverse transform (see msosm_persist.cu).
#pragma once
#include "msosm_kernels.cuh"

namespace msosm {

struct PersistArgs
{
    const float2 *ring;
    const float2 *H;
    const uint16_t *delays;
    float2 *T;       // S slots of F complex values
    int S, lag;      // ring slots of T and the P2 look-behind in transforms
    int rbi, fbs, B;
    long long g0, G; // transforms g0 .. g0+G-1 (g = d*B + b)
    Twiddles tw;     // inverse direction
    int out_mode;
    float2 *out_c64;
    uint32_t *out_u16;
    float *out_pow;        // OUT_POW: |x|^2 per output sample
    const float *pair_pow; // OUT_PAIR: the other polarisation's |a|^2, same layout
    FoldArgs fold;
    unsigned *ticket;  // zeroed before the launch
    unsigned *p1_done; // [S], zeroed before the launch
    unsigned *p2_done; // [S], zeroed before the launch
    int *err;          // sticky error flag (1 = a wait timed out)
    unsigned long long timeout_ns;
    int max_ctas_per_sm; // host side: cap on resident CTAs per SM of the launch (0 = as many as fit)
    // transform order: groups of dm_group DM trials, window-major inside a group, so that
    // consecutive transforms read the same ring slots (D = number of DM trials)
    int D, dm_group;
};

// Split-precision transform (tensor cores): precisions and extra arguments.
enum Precision : int
{
    PREC_FP32 = 0,   // FP32 register transform (the plain form)
    PREC_BF16X3 = 1, // DFT contractions on BF16 hi/lo operands, FP32 accumulation
    PREC_FP16X3 = 2, // the same on FP16 hi/lo operands, power-of-two operand scaling
};

struct TcArgs
{
    const uint4 *bop;       // W_32 operand image: hi (8 KB) then lo (8 KB), K-major 128-byte swizzled
    const unsigned *absmax; // FP16: running max |component| over the spectra ring (float bits)
    float hmax;             // FP16: max |H| over the DM trials
};

struct PersistPlan
{
    int lag = 0, slots = 0, grid = 0;
    int occupancy = 0; // CTAs per SM the occupancy query reported
};

bool persist_supported(int L);
// Return persisting L2 lines to normal and the persisting set-aside to zero (the next
// persistent launch sets it again for its slot ring).
cudaError_t persist_l2_reset();
// The persistent kernel's bounded wait, run alone (see msosm_selftest_wait).
cudaError_t persist_selftest_wait(unsigned preset, unsigned target, unsigned long long timeout_ns, int *timed_out,
                                  unsigned long long *elapsed_ns);
// Grid and ring geometry for the given sizes / output mode (no launch).
cudaError_t persist_plan(int L, const PersistArgs &a, int sms, PersistPlan *plan);
cudaError_t launch_inverse_persistent(int L, const PersistArgs &a, int sms, cudaStream_t st);

// Split-precision persistent transform (F = 2^18 only).
bool tc_supported(int L);
cudaError_t tc_plan(int L, int prec, const PersistArgs &a, const TcArgs &tc, int sms, PersistPlan *plan);
cudaError_t launch_inverse_tc(int L, int prec, const PersistArgs &a, const TcArgs &tc, int sms, cudaStream_t st);

} // namespace msosm
