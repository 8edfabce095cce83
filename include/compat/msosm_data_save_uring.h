// Drop-in replacement for data_save/include/msosm_data_save_uring.h (header-only).
//
// MSOSM_DataSave_Uring with the reference's constructor and methods
// (msosm_data_save_uring.h:22-52) over the engine's per-DM writer (msosm_writer_*):
//   config_save(dir, prefix)           the output directory and file prefix; files
//                                      <dir>/<prefix>_DM<value>.dat, decimals chosen as
//                                      the reference does (msosm_data_save_uring.cpp:40-71)
//   initialize_uring(slots, count)     `slots` page-aligned host slots of one step's
//                                      [DM][B*M] uint16 pairs (:73-98)
//   copy_to_slot()                     the last step's output into a free slot (:100-110)
//   start_saving() / join_saving()     the writer's worker threads write each slot's DM
//                                      blocks at the step's file offset with pwrite
//                                      (O_DIRECT when the file system accepts it); join
//                                      waits until every copied step is on disk (:112-288)
// poll_cuda_state / save_to_disk / save_to_disk_pwrite exist for source compatibility;
// the writer's workers do their work.  No liburing is needed.
#pragma once
#include "globals.h"
#include "msosm_gpu_batch.h"

#include <atomic>
#include <fcntl.h>
#include <iomanip>
#include <string>
#include <unistd.h>

enum class SaveSlotState
{
    EMPTY,
    COPYING,
    READY,
    SAVING,
    DONE
};

class MSOSM_DataSave_Uring : public MSOSM_GPU_BATCH
{
  public:
    MSOSM_DataSave_Uring(float bw, float *dm, float f0, int numDMs) : MSOSM_GPU_BATCH(bw, dm, f0, numDMs) {}
    ~MSOSM_DataSave_Uring() override
    {
        if (w)
        {
            msosm_writer_join(w);
            msosm_writer_destroy(w);
            w = nullptr;
        }
    }

    void config_save(string dir = "", string prefix = "")
    {
        save_dir = dir.empty() ? "." : dir;
        save_prefix = prefix;
    }
    void initialize_uring(int slot_count, unsigned long save_count)
    {
        this->slot_count = slot_count;
        this->save_count = save_count;
        const unsigned long long per_dm = (unsigned long long)batch * (unsigned long long)M * sizeof(uint16_pair);
        const int rc = msosm_writer_create(save_dir.c_str(), save_prefix.c_str(), dm_values, numDMs, per_dm, slot_count,
                                           1, &w);
        if (rc != MSOSM_OK)
        {
            cerr << "FATAL: writer creation failed: " << msosm_status_string(rc) << endl;
            exit(1);
        }
    }
    void copy_to_slot()
    {
        if (copied >= save_count)
            return; // the reference's poll thread stops after save_count slots
        msosm_compat::check(msosm_writer_copy_output(w, h, nullptr), h, "copy_to_slot");
        copied++;
    }
    void poll_cuda_state() {}
    void save_to_disk(int) {}
    void save_to_disk_pwrite(int) {}
    void start_saving() {}
    void join_saving()
    {
        if (!w)
            return;
        const int rc = msosm_writer_join(w);
        if (rc != MSOSM_OK)
        {
            cerr << "FATAL: " << msosm_writer_last_error(w) << endl;
            exit(1);
        }
    }

  private:
    unsigned long save_count = 0;
    unsigned long copied = 0;
    int slot_count = 0;
    string save_dir = ".";
    string save_prefix;
    msosm_writer_t *w = nullptr;
};
