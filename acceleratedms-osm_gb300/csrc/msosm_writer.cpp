// Per-DM output files: the reference's data_save front end
// (data_save/msosm_data_save_uring.cpp:40-288, MSOSM_DataSave_Uring) rebuilt on
// pwrite worker threads, since liburing is not available everywhere.
//
// Same pipeline shape: a ring of `slots` page-aligned host buffers (pinned when a
// GPU is present); a step's [D][bytes_per_dm] output is copied device->host into a
// free slot on the caller's stream with an event behind it (copy_to_slot, :103-113);
// a worker waits for that event (poll_cuda_state, :115-154) and writes each DM's
// part at offset step * bytes_per_dm of that DM's file (save_to_disk_pwrite,
// :224-258), then frees the slot.  One file per DM, named as config_save names
// them (:40-71): <dir>/<prefix>_DM<value>.dat with the reference's choice of
// decimals.  The data is the uint16-pair stream python_check/check.py reads.
#include "msosm_gb300.h"
#include "msosm_writer.h"

#include <cuda_runtime.h>

#include <algorithm>
#include <cerrno>
#include <cmath>
#include <condition_variable>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <deque>
#include <fcntl.h>
#include <mutex>
#include <new>
#include <sstream>
#include <string>
#include <thread>
#include <unistd.h>
#include <vector>

namespace {

// get_decimal_places_from_dm (msosm_data_save_uring.cpp:16-40): the fewest
// decimals that print dm exactly at float precision; integers get 2, DM 0 gets 0.
int decimal_places(float dm, int max_places = 10)
{
    dm = std::fabs(dm);
    if (dm <= 0.0f)
        return 0;
    int ret = max_places;
    for (int places = 0; places <= max_places; ++places)
    {
        const float scaled = (float)(dm * std::pow(10.0, places));
        const float rounded = std::round(scaled);
        if (std::fabs(scaled - rounded) < 1e-6)
        {
            ret = places;
            break;
        }
    }
    if (ret == 0)
        ret = 2;
    return ret;
}

struct Job
{
    int slot;
    long long index;
    bool device;
};

} // namespace

struct msosm_writer_s
{
    std::vector<std::string> names;
    std::vector<int> fds;
    size_t bytes_per_dm = 0;
    int D = 0;
    std::vector<char *> slots;
    std::vector<bool> pinned;
    std::vector<cudaEvent_t> events;
    std::mutex mu;
    std::condition_variable cv;
    std::deque<Job> queue;
    std::vector<int> free_slots;
    long long next_index = 0;
    long long outstanding = 0;
    bool stop = false;
    std::vector<std::thread> workers;
    int err_code = MSOSM_OK;
    std::string err;

    void fail(int code, const std::string &m)
    {
        std::lock_guard<std::mutex> l(mu);
        if (err_code == MSOSM_OK)
        {
            err_code = code;
            err = m;
        }
    }

    void worker()
    {
        for (;;)
        {
            Job j;
            {
                std::unique_lock<std::mutex> l(mu);
                cv.wait(l, [&] { return stop || !queue.empty(); });
                if (queue.empty())
                    return;
                j = queue.front();
                queue.pop_front();
            }
            bool ok = true;
            if (j.device)
            {
                cudaError_t e = cudaEventSynchronize(events[j.slot]);
                if (e != cudaSuccess)
                {
                    fail(MSOSM_ERR_CUDA, std::string("writer: ") + cudaGetErrorString(e));
                    ok = false;
                }
            }
            for (int d = 0; ok && d < D; d++)
            {
                const char *p = slots[j.slot] + (size_t)d * bytes_per_dm;
                size_t left = bytes_per_dm;
                off_t off = (off_t)((unsigned long long)j.index * bytes_per_dm);
                while (left > 0)
                {
                    const ssize_t n = pwrite(fds[d], p, left, off);
                    if (n < 0 && errno == EINTR)
                        continue;
                    if (n <= 0)
                    {
                        fail(MSOSM_ERR_ARG, "writer: pwrite " + names[d] + ": " + std::strerror(errno));
                        ok = false;
                        break;
                    }
                    p += n;
                    off += n;
                    left -= (size_t)n;
                }
            }
            {
                std::lock_guard<std::mutex> l(mu);
                free_slots.push_back(j.slot);
                outstanding--;
            }
            cv.notify_all();
        }
    }

    int acquire_slot()
    {
        std::unique_lock<std::mutex> l(mu);
        cv.wait(l, [&] { return !free_slots.empty(); });
        const int s = free_slots.back();
        free_slots.pop_back();
        return s;
    }

    void enqueue(int slot, bool device)
    {
        {
            std::lock_guard<std::mutex> l(mu);
            queue.push_back({slot, next_index++, device});
            outstanding++;
        }
        cv.notify_all();
    }

    void join()
    {
        std::unique_lock<std::mutex> l(mu);
        cv.wait(l, [&] { return outstanding == 0; });
    }

    ~msosm_writer_s()
    {
        join();
        {
            std::lock_guard<std::mutex> l(mu);
            stop = true;
        }
        cv.notify_all();
        for (auto &t : workers)
            t.join();
        for (int fd : fds)
            if (fd >= 0)
                close(fd);
        for (size_t i = 0; i < slots.size(); i++)
        {
            if (pinned[i])
                cudaHostUnregister(slots[i]);
            std::free(slots[i]);
        }
        for (auto e : events)
            if (e)
                cudaEventDestroy(e);
    }
};

namespace msosm {

int writer_submit_device(msosm_writer_s *w, const void *dev, cudaStream_t st, std::string &err)
{
    const int s = w->acquire_slot();
    if (!w->events[s] && cudaEventCreateWithFlags(&w->events[s], cudaEventDisableTiming) != cudaSuccess)
    {
        err = "writer: cudaEventCreate failed";
        std::lock_guard<std::mutex> l(w->mu);
        w->free_slots.push_back(s);
        return MSOSM_ERR_CUDA;
    }
    cudaError_t e = cudaMemcpyAsync(w->slots[s], dev, w->bytes_per_dm * w->D, cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess)
        e = cudaEventRecord(w->events[s], st);
    if (e != cudaSuccess)
    {
        err = std::string("writer: ") + cudaGetErrorString(e);
        std::lock_guard<std::mutex> l(w->mu);
        w->free_slots.push_back(s);
        return MSOSM_ERR_CUDA;
    }
    w->enqueue(s, true);
    return MSOSM_OK;
}

size_t writer_bytes_per_step(const msosm_writer_s *w) { return w->bytes_per_dm * (size_t)w->D; }
int writer_num_files(const msosm_writer_s *w) { return w->D; }

} // namespace msosm

extern "C" int msosm_writer_create(const char *dir, const char *prefix, const float *dms, int num_dms,
                                   unsigned long long bytes_per_dm, int slots, int direct_io, msosm_writer_t **out)
{
    if (!out || !dms || num_dms <= 0 || bytes_per_dm == 0 || slots <= 0 || slots > 64)
        return MSOSM_ERR_ARG;
    *out = nullptr;
    msosm_writer_s *w = new (std::nothrow) msosm_writer_s();
    if (!w)
        return MSOSM_ERR_NOMEM;
    w->D = num_dms;
    w->bytes_per_dm = (size_t)bytes_per_dm;
    const std::string d = (dir && *dir) ? dir : ".";
    const std::string pre = (prefix && *prefix) ? std::string(prefix) + "_" : "";
    int prec = decimal_places(dms[0], 10);
    if (num_dms > 1)
        prec = std::max(prec, decimal_places(dms[1], 10));
    const bool aligned = (bytes_per_dm % 4096) == 0;
    for (int i = 0; i < num_dms; i++)
    {
        std::ostringstream oss;
        oss.setf(std::ios::fixed);
        oss.precision(prec);
        oss << d << "/" << pre << "DM" << (double)dms[i] << ".dat";
        w->names.push_back(oss.str());
        int fd = -1;
        if (direct_io && aligned)
            fd = open(w->names.back().c_str(), O_WRONLY | O_CREAT | O_TRUNC | O_DIRECT, 0644);
        if (fd < 0) // O_DIRECT unsupported here (e.g. tmpfs) or not requested
            fd = open(w->names.back().c_str(), O_WRONLY | O_CREAT | O_TRUNC, 0644);
        if (fd < 0)
        {
            delete w;
            return MSOSM_ERR_ARG;
        }
        w->fds.push_back(fd);
    }
    const size_t slot_bytes = w->bytes_per_dm * (size_t)num_dms;
    for (int s = 0; s < slots; s++)
    {
        void *p = nullptr;
        if (posix_memalign(&p, 4096, slot_bytes) != 0)
        {
            delete w;
            return MSOSM_ERR_NOMEM;
        }
        w->slots.push_back(static_cast<char *>(p));
        // pinned when a GPU is present, so device->host copies are asynchronous
        const bool pin = cudaHostRegister(p, slot_bytes, cudaHostRegisterDefault) == cudaSuccess;
        if (!pin)
            cudaGetLastError();
        w->pinned.push_back(pin);
        w->events.push_back(nullptr);
        w->free_slots.push_back(s);
    }
    for (int s = 0; s < slots; s++)
        w->workers.emplace_back(&msosm_writer_s::worker, w);
    *out = w;
    return MSOSM_OK;
}

extern "C" int msosm_writer_write(msosm_writer_t *w, const void *host_block)
{
    if (!w || !host_block)
        return MSOSM_ERR_ARG;
    const int s = w->acquire_slot();
    std::memcpy(w->slots[s], host_block, w->bytes_per_dm * (size_t)w->D);
    w->enqueue(s, false);
    return MSOSM_OK;
}

extern "C" int msosm_writer_join(msosm_writer_t *w)
{
    if (!w)
        return MSOSM_ERR_ARG;
    w->join();
    std::lock_guard<std::mutex> l(w->mu);
    return w->err_code;
}

extern "C" const char *msosm_writer_last_error(const msosm_writer_t *w) { return w ? w->err.c_str() : "null writer"; }

extern "C" int msosm_writer_filename(const msosm_writer_t *w, int dm_index, char *buf, size_t len)
{
    if (!w || !buf || dm_index < 0 || dm_index >= w->D || len == 0)
        return MSOSM_ERR_ARG;
    std::snprintf(buf, len, "%s", w->names[dm_index].c_str());
    return w->names[dm_index].size() < len ? MSOSM_OK : MSOSM_ERR_ARG;
}

extern "C" int msosm_writer_destroy(msosm_writer_t *w)
{
    if (!w)
        return MSOSM_ERR_ARG;
    delete w;
    return MSOSM_OK;
}
