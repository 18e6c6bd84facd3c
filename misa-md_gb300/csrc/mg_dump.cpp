// Atom dump writer: the copy-mode binary dump of frontend/io (AtomDump, frontend/io/atom_dump.cpp:38-82;
// OutputCopy, frontend/io/output_copy.cpp:19-59) fed from device buffers.
//
// File layout for one rank, as tools/dump2text/out_convert.cpp:66-98 reads it: 128 bytes of file
// header (kiwi::LocalStorage's; zeros here), a 128-byte rank header whose first 8 bytes are the
// record count (AtomDump::writeDumpHeader, atom_dump.cpp:77-82), then 72-byte records. With one rank
// the 1024-record blocks of LocalStorage follow each other, so the records are contiguous.
//
// A frame is packed on the device into one of two staging buffers (the caller's stream). A writer
// thread waits for the pack, reads the record count, and moves the records through two pinned chunks
// on its own stream: the copy of chunk k + 1 runs while chunk k is written to the file.
#include <algorithm>
#include <condition_variable>
#include <cstdio>
#include <cstring>
#include <deque>
#include <mutex>
#include <string>
#include <thread>

#include "mg_internal.h"

using namespace mg;

namespace {
constexpr int64_t kHeaderBytes = 128;       // HEADER_SIZE, out_convert.cpp:5
constexpr int64_t kRankHeaderBytes = 128;   // _LOCAL_HEADER_SIZE, out_convert.cpp:6
constexpr int64_t kDefaultChunk = 64ll << 20;

struct Job {
    int slot;
    uint64_t step;
};
}  // namespace

struct mg_dump {
    mg_context *ctx = nullptr;
    std::string path;
    bool by_frame = false;
    FILE *file = nullptr;               // single-file mode
    uint64_t records = 0;               // written so far (all frames)
    int64_t max_records = 0;
    int64_t chunk = kDefaultChunk;
    cudaStream_t stream = nullptr;      // the context's stream (packs)
    cudaStream_t io = nullptr;          // the writer's copies
    mg_dump_record *stage[2] = {nullptr, nullptr};
    unsigned long long *d_count = nullptr;  // [2]
    int *scratch = nullptr;
    cudaEvent_t packed[2] = {nullptr, nullptr};
    cudaEvent_t copied[2] = {nullptr, nullptr};
    unsigned char *pin[2] = {nullptr, nullptr};
    unsigned long long *h_count = nullptr;
    bool busy[2] = {false, false};
    int next = 0;
    int device = 0;
    std::thread writer;
    mutable std::mutex mu;
    std::condition_variable cv;
    std::deque<Job> queue;
    bool stop = false;
    mg_status failed = MG_OK;           // first failure of the writer
    std::string err;

    void fail(mg_status st, const std::string &why) {
        std::lock_guard<std::mutex> lk(mu);
        if (failed == MG_OK) { failed = st; err = why; }
    }
    std::string frame_path(uint64_t step) const {  // fmt::format(path, step) with one "{}"
        const size_t at = path.find("{}");
        return path.substr(0, at) + std::to_string(step) + path.substr(at + 2);
    }
    bool write_header(FILE *f, uint64_t n) {
        unsigned char h[kHeaderBytes + kRankHeaderBytes];
        std::memset(h, 0, sizeof(h));
        std::memcpy(h + kHeaderBytes, &n, sizeof(n));  // struct { size_t atoms_count; }
        return std::fseek(f, 0, SEEK_SET) == 0 && std::fwrite(h, 1, sizeof(h), f) == sizeof(h);
    }
    // one frame: count, then the records through the pinned chunks
    void write_frame(const Job &j) {
        if (cudaEventSynchronize(packed[j.slot]) != cudaSuccess ||
            cudaMemcpyAsync(h_count, d_count + j.slot, sizeof(unsigned long long), cudaMemcpyDeviceToHost, io) != cudaSuccess ||
            cudaStreamSynchronize(io) != cudaSuccess) {
            fail(MG_ERR_CUDA, std::string("dump copy: ") + cudaGetErrorString(cudaGetLastError()));
            return;
        }
        const uint64_t n = *h_count;
        FILE *f = file;
        std::string fp;
        if (by_frame) {
            fp = frame_path(j.step);
            f = std::fopen(fp.c_str(), "wb");
            if (!f || !write_header(f, n)) {
                if (f) std::fclose(f);
                fail(MG_ERR_ARG, "cannot write " + fp);
                return;
            }
        }
        const int64_t bytes = static_cast<int64_t>(n) * static_cast<int64_t>(sizeof(mg_dump_record));
        const unsigned char *src = reinterpret_cast<const unsigned char *>(stage[j.slot]);
        bool ok = true;
        int64_t prev_len = -1;
        int prev = 0, k = 0;
        for (int64_t off = 0; off < bytes && ok; off += chunk, k ^= 1) {
            const int64_t len = std::min(chunk, bytes - off);
            if (cudaMemcpyAsync(pin[k], src + off, static_cast<size_t>(len), cudaMemcpyDeviceToHost, io) != cudaSuccess ||
                cudaEventRecord(copied[k], io) != cudaSuccess) {
                ok = false;
                break;
            }
            if (prev_len >= 0) {  // chunk k is in flight: write the previous one
                ok = cudaEventSynchronize(copied[prev]) == cudaSuccess &&
                     std::fwrite(pin[prev], 1, static_cast<size_t>(prev_len), f) == static_cast<size_t>(prev_len);
            }
            prev = k;
            prev_len = len;
        }
        if (ok && prev_len >= 0)
            ok = cudaEventSynchronize(copied[prev]) == cudaSuccess &&
                 std::fwrite(pin[prev], 1, static_cast<size_t>(prev_len), f) == static_cast<size_t>(prev_len);
        if (by_frame) ok = (std::fclose(f) == 0) && ok;
        if (!ok) {
            fail(MG_ERR_ARG, "dump write failed: " + (by_frame ? fp : path));
            return;
        }
        std::lock_guard<std::mutex> lk(mu);
        records += n;
    }
    void run() {
        cudaSetDevice(device);
        for (;;) {
            Job j;
            {
                std::unique_lock<std::mutex> lk(mu);
                cv.wait(lk, [&] { return stop || !queue.empty(); });
                if (queue.empty()) return;  // stop requested and nothing left
                j = queue.front();
            }
            bool skip;
            {
                std::lock_guard<std::mutex> lk(mu);
                skip = failed != MG_OK;
            }
            if (!skip) write_frame(j);
            {
                std::lock_guard<std::mutex> lk(mu);
                queue.pop_front();
                busy[j.slot] = false;
            }
            cv.notify_all();
        }
    }
    void release() {
        for (int k = 0; k < 2; k++) {
            if (stage[k]) cudaFree(stage[k]);
            if (packed[k]) cudaEventDestroy(packed[k]);
            if (copied[k]) cudaEventDestroy(copied[k]);
            if (pin[k]) cudaFreeHost(pin[k]);
        }
        if (d_count) cudaFree(d_count);
        if (scratch) cudaFree(scratch);
        if (h_count) cudaFreeHost(h_count);
        if (io) cudaStreamDestroy(io);
        if (file) std::fclose(file);
    }
};

extern "C" {

mg_status mg_dump_open(mg_context *ctx, const char *path, int32_t by_frame, int64_t chunk_bytes, mg_dump **out) {
    if (!ctx || !path || !out || chunk_bytes < 0) return MG_ERR_ARG;
    *out = nullptr;
    auto *d = new mg_dump();
    d->ctx = ctx;
    d->path = path;
    d->by_frame = by_frame != 0;
    if (chunk_bytes > 0) d->chunk = chunk_bytes;
    if (d->by_frame && d->path.find("{}") == std::string::npos) {  // config_parser.cpp:208-210
        delete d;
        return MG_ERR_ARG;
    }
    const DumpSource src = dump_source(ctx);
    d->stream = src.stream;
    d->max_records = src.max_records;
    const size_t frame_bytes = static_cast<size_t>(src.max_records) * sizeof(mg_dump_record);
    const size_t pin_bytes = static_cast<size_t>(std::min<int64_t>(d->chunk, static_cast<int64_t>(frame_bytes)));
    bool ok = cudaStreamCreateWithFlags(&d->io, cudaStreamNonBlocking) == cudaSuccess &&
              cudaMalloc(&d->d_count, 2 * sizeof(unsigned long long)) == cudaSuccess &&
              cudaMalloc(&d->scratch, static_cast<size_t>(src.scratch_ints) * sizeof(int)) == cudaSuccess &&
              cudaHostAlloc(&d->h_count, sizeof(unsigned long long), cudaHostAllocDefault) == cudaSuccess;
    for (int k = 0; k < 2 && ok; k++) {
        ok = cudaMalloc(&d->stage[k], frame_bytes) == cudaSuccess &&
             cudaEventCreateWithFlags(&d->packed[k], cudaEventDisableTiming) == cudaSuccess &&
             cudaEventCreateWithFlags(&d->copied[k], cudaEventDisableTiming) == cudaSuccess &&
             cudaHostAlloc(&d->pin[k], pin_bytes, cudaHostAllocDefault) == cudaSuccess;
    }
    if (!ok) {
        d->release();
        delete d;
        return MG_ERR_CUDA;
    }
    if (!d->by_frame) {
        d->file = std::fopen(path, "wb");
        if (!d->file || !d->write_header(d->file, 0)) {
            d->release();
            delete d;
            return MG_ERR_ARG;
        }
    }
    cudaGetDevice(&d->device);
    try {
        d->writer = std::thread([d] { d->run(); });
    } catch (...) {
        d->release();
        delete d;
        return MG_ERR_STATE;
    }
    *out = d;
    return MG_OK;
}

mg_status mg_dump_frame(mg_dump *d, uint64_t time_step) {
    if (!d) return MG_ERR_ARG;
    int slot;
    {
        std::unique_lock<std::mutex> lk(d->mu);
        if (d->failed != MG_OK) return d->failed;
        slot = d->next;
        d->cv.wait(lk, [&] { return !d->busy[slot] || d->failed != MG_OK; });
        if (d->failed != MG_OK) return d->failed;
    }
    mg_status st = dump_pack(d->ctx, d->stage[slot], d->d_count + slot, d->scratch, time_step);
    if (st == MG_OK && cudaEventRecord(d->packed[slot], d->stream) != cudaSuccess) st = MG_ERR_CUDA;
    if (st != MG_OK) {
        d->fail(st, "dump pack failed: " + std::string(mg_last_error(d->ctx)));
        return st;
    }
    {
        std::lock_guard<std::mutex> lk(d->mu);
        d->busy[slot] = true;
        d->queue.push_back(Job{slot, time_step});
        d->next = slot ^ 1;
    }
    d->cv.notify_all();
    return MG_OK;
}

mg_status mg_dump_close(mg_dump *d, uint64_t *records) {
    if (!d) return MG_ERR_ARG;
    {
        std::lock_guard<std::mutex> lk(d->mu);
        d->stop = true;
    }
    d->cv.notify_all();
    d->writer.join();
    dump_detach(d->ctx, d);
    mg_status st = d->failed;
    if (d->file) {
        // OutputCopy::onAllOut -> AtomDump::writeDumpHeader: the count of every record in the file
        const bool ok = d->write_header(d->file, d->records);
        const bool closed = std::fclose(d->file) == 0;
        d->file = nullptr;
        if (st == MG_OK && !(ok && closed)) st = MG_ERR_ARG;
    }
    if (records) *records = d->records;
    if (st != MG_OK) dump_note_error(d->ctx, d->err.empty() ? "dump: cannot write the header of " + d->path : d->err);
    d->release();
    delete d;
    return st;
}

const char *mg_dump_last_error(const mg_dump *d) {
    if (!d) return "null dump";
    std::lock_guard<std::mutex> lk(d->mu);  // set once, by the first failure
    return d->err.c_str();
}

}  // extern "C"
