// Per-DM output writer (internal interface between the C ABI and the writer).
#pragma once
#include <cuda_runtime.h>

#include <string>

struct msosm_writer_s;

namespace msosm {
// Queue the D2H copy of one step's [D][bytes_per_dm] output from device memory on
// `st`, then its per-DM pwrite on a worker thread.  Blocks while every slot is busy.
int writer_submit_device(msosm_writer_s *w, const void *dev, cudaStream_t st, std::string &err);
size_t writer_bytes_per_step(const msosm_writer_s *w);
int writer_num_files(const msosm_writer_s *w);
} // namespace msosm
