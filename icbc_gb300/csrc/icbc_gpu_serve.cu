// icbc_gpu_serve.cu -- the serving form: continuous batching of encode requests.
//
// A scheduler thread owns the GPU side.  Requests wait in a FIFO until their
// texels and blocks fit in the device arena (allocated once, at create); the
// admitted ones are gathered into the next batched launch (the persistent
// kernel of bc1_batch.cu, one task list per launch), which runs on one of
// max_inflight streams -- so requests that arrive while a batch runs are
// admitted as arena space frees up and their batch overlaps the running one
// (copies on one stream run under another stream's kernel).  Each launch
// copies its blocks to pinned staging; a host callback marks the launch done,
// the scheduler frees its device space and slot, and a delivery thread hands
// the blocks to the callers' buffers (host copies off the scheduler's path)
// and frees the staging.  No waits on the device side: the kernel drains a
// finite queue.
// A launch runs in the batched form's two passes: the blocks of 0 or 1
// reduced colours of level-2..9 requests are finished by a register-only
// pass, which lists the others in the request's own arena space.
// Light requests (under ~0.2 ms of GPU time) and heavy ones go to separate
// launches -- light first, the two in turn while both wait -- because a
// launch completes as a whole, so a small request batched with a large one
// would wait for it; and a launch with more tasks than the GPU has CTA slots
// takes three quarters of them, so launches behind it start on the rest.
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <map>
#include <mutex>
#include <thread>
#include <unordered_map>
#include <utility>
#include <vector>

#include "../../include/icbc_gpu.h"
#include "bc1_kernels.h"

namespace icbc_gpu {
namespace {

constexpr size_t kGranule = 256;

size_t round_up(size_t x, size_t a) { return (x + a - 1) / a * a; }

double now_ms() {
    return std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

// First-fit allocator over offsets [0, size), coalescing freed ranges.
class Arena {
  public:
    void reset(size_t size) {
        free_.clear();
        size_ = size;
        used_ = 0;
        if (size) free_[0] = size;
    }
    bool alloc(size_t bytes, size_t *off) {
        bytes = round_up(bytes ? bytes : 1, kGranule);
        for (auto it = free_.begin(); it != free_.end(); ++it) {
            if (it->second >= bytes) {
                *off = it->first;
                const size_t rest = it->second - bytes, tail = it->first + bytes;
                free_.erase(it);
                if (rest) free_[tail] = rest;
                used_ += bytes;
                return true;
            }
        }
        return false;
    }
    void release(size_t off, size_t bytes) {
        bytes = round_up(bytes ? bytes : 1, kGranule);
        used_ -= bytes;
        auto next = free_.lower_bound(off);
        if (next != free_.begin()) {
            auto prev = std::prev(next);
            if (prev->first + prev->second == off) {
                off = prev->first;
                bytes += prev->second;
                free_.erase(prev);
            }
        }
        if (next != free_.end() && off + bytes == next->first) {
            bytes += next->second;
            free_.erase(next);
        }
        free_[off] = bytes;
    }
    size_t size() const { return size_; }
    size_t used() const { return used_; }

  private:
    std::map<size_t, size_t> free_;
    size_t size_ = 0, used_ = 0;
};

struct Request {
    uint64_t id = 0;
    icbc_gpu_request r{};
    ImageDesc d{};
    int64_t dpitch = 0;
    size_t dev_off = 0, dev_bytes = 0, out_off = 0, err_off = 0, list_off = 0;
    size_t host_off = 0, host_bytes = 0;
    size_t in_off = 0, in_bytes = 0;  // pinned copy of the texels (rows at dpitch), then at levels 4-9 the
                                      // zero blocks the encoder starts from, laid out as on the device
    bool staged = false;
    bool heavy = false;  // about 0.2 ms of GPU time or more (heavy_request)
    double t_submit = 0.0;
};

struct Slot {
    cudaStream_t stream = nullptr;
    ImageDesc *d_images = nullptr;
    uint32_t *d_start = nullptr;
    int *d_counter = nullptr;
    ImageDesc *h_images = nullptr;   // pinned
    uint32_t *h_start = nullptr;     // pinned
    // Two passes: each request's list (base in 4-byte entries from the arena
    // start; -1 below level 2) and its count.
    int64_t *d_list_base = nullptr;
    int64_t *h_list_base = nullptr;  // pinned
    unsigned int *d_listed = nullptr;
    std::vector<Request *> reqs;
    bool busy = false;
    int status = ICBC_GPU_OK;
    std::atomic<bool> done{false};
    std::condition_variable *wake = nullptr;  // the scheduler's
};

}  // namespace
}  // namespace icbc_gpu

using namespace icbc_gpu;

struct icbc_gpu_server {
    icbc_gpu_server_config cfg{};
    int device = 0;
    const GlobalTables *G = nullptr;
    int grid = 1;
    uint8_t *d_arena = nullptr;
    uint8_t *h_stage = nullptr;
    uint8_t *h_in = nullptr;  // pinned input staging, filled by submit() on the caller's thread
    Arena dev, host, in;
    std::vector<Slot> slots;
    std::mutex m;
    std::condition_variable cv_work, cv_done;
    std::deque<Request *> pending, admitted;
    bool heavy_turn = false;  // light and heavy launches alternate while both wait
    // Finished launches (requests, status) waiting for their host copies.
    std::deque<std::pair<std::vector<Request *>, int>> delivery;
    std::condition_variable cv_deliver;
    std::thread deliverer;
    bool scheduler_done = false;
    std::unordered_map<uint64_t, Request *> live;
    std::unordered_map<uint64_t, int> finished;
    std::vector<double> latencies;
    std::thread worker;
    bool stop = false;
    uint64_t next_id = 1;
    int64_t submitted = 0, completed = 0, rejected = 0, cancelled = 0, failed = 0, batches = 0;
    int64_t arena_peak = 0;
    double pixels = 0.0;
    int in_flight = 0;
};

namespace {

// Whether a request alone takes about 0.2 ms of GPU time or more: blocks
// times the encoder's nanoseconds per block at its level on a GB300 (the
// quality-sweep image, a whole GPU).
bool heavy_request(const ImageDesc &d) {
    static const double kBlockNs[10] = {0.09, 0.15, 0.11, 0.12, 0.19, 0.38, 0.65, 1.0, 3.7, 4.5};
    return (double)d.nblocks * kBlockNs[d.level < 0 ? 0 : d.level > 9 ? 9 : d.level] >= 2.0e5;
}

// Device and pinned bytes a request needs.
void size_request(icbc_gpu_server *S, Request *q) {
    const int64_t nb = (int64_t)((q->r.width + 3) / 4) * ((q->r.height + 3) / 4);
    q->dpitch = (int64_t)round_up(4 * (size_t)q->r.width, 16);
    const size_t img = round_up((size_t)q->dpitch * q->r.height, kGranule);
    const size_t out = round_up((size_t)nb * 8, kGranule);
    const size_t err = q->r.errors ? round_up((size_t)nb * 4, kGranule) : 0;
    const size_t list = q->d.level >= 2 ? round_up((size_t)nb * 4, kGranule) : 0;
    q->list_off = img + out + err;
    q->dev_bytes = img + out + err + list;
    q->host_bytes = out + err;
    (void)S;
}

// Runs on a CUDA callback thread after the slot's last copy: no CUDA calls.
void CUDART_CB on_slot_done(void *arg) {
    Slot *slot = static_cast<Slot *>(arg);
    slot->done.store(true, std::memory_order_release);
    slot->wake->notify_one();
}

// Stages a batch of admitted requests and launches it on a free slot.
// Called by the scheduler without the lock held.
int launch_slot(icbc_gpu_server *S, Slot &slot) {
    std::vector<Request *> &reqs = slot.reqs;
    std::stable_sort(reqs.begin(), reqs.end(), [](const Request *a, const Request *b) {
        return level_cost(a->r.level) > level_cost(b->r.level);
    });
    cudaError_t e = cudaSuccess;
    uint32_t total = 0, listed_tasks = 0;  // level-2..9 requests come first: their tasks lead
    for (size_t i = 0; i < reqs.size() && e == cudaSuccess; i++) {
        Request *q = reqs[i];
        uint8_t *base = S->d_arena + q->dev_off;
        ImageDesc d = q->d;
        d.rgba = base;
        d.pitch = q->dpitch;
        d.vec16 = 1;
        d.out = reinterpret_cast<uint2 *>(base + q->out_off);
        d.errors = q->r.errors ? reinterpret_cast<float *>(base + q->err_off) : nullptr;
        if (q->staged)
            e = cudaMemcpyAsync(base, S->h_in + q->in_off, q->in_bytes, cudaMemcpyHostToDevice, slot.stream);
        else
            e = cudaMemcpy2DAsync(base, (size_t)q->dpitch, q->r.rgba, (size_t)q->r.pitch, 4 * (size_t)q->r.width,
                                  (size_t)q->r.height, cudaMemcpyHostToDevice, slot.stream);
        if (e == cudaSuccess && d.level >= 4 && !q->staged)
            e = cudaMemsetAsync(d.out, 0, (size_t)d.nblocks * 8, slot.stream);
        slot.h_images[i] = d;
        slot.h_start[i] = total;
        slot.h_list_base[i] = d.level >= 2 && d.nblocks > 0 ? (int64_t)((q->dev_off + q->list_off) / 4) : -1;
        if (d.level >= 2) listed_tasks = total + (uint32_t)((d.nblocks + 31) / 32);
        total += (uint32_t)((d.nblocks + 31) / 32);
    }
    slot.h_start[reqs.size()] = total;
    const int n = (int)reqs.size();
    const BatchLists lists{reinterpret_cast<uint32_t *>(S->d_arena), slot.d_listed, slot.d_list_base};
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(slot.d_images, slot.h_images, sizeof(ImageDesc) * n, cudaMemcpyHostToDevice, slot.stream);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(slot.d_start, slot.h_start, sizeof(uint32_t) * (n + 1), cudaMemcpyHostToDevice,
                            slot.stream);
    if (e == cudaSuccess) e = cudaMemsetAsync(slot.d_counter, 0, sizeof(int), slot.stream);
    if (e == cudaSuccess && listed_tasks) {
        e = cudaMemcpyAsync(slot.d_list_base, slot.h_list_base, sizeof(int64_t) * n, cudaMemcpyHostToDevice,
                            slot.stream);
        if (e == cudaSuccess) e = cudaMemsetAsync(slot.d_listed, 0, sizeof(unsigned int) * n, slot.stream);
        if (e == cudaSuccess)
            e = launch_batch_trivial(S->G, slot.d_images, nullptr, slot.d_start, n, (int)listed_tasks, lists, nullptr,
                                     nullptr, slot.stream, current_sm_count());
    }
    if (e == cudaSuccess) {
        // A persistent grid no larger than the batch's work (four tasks per
        // CTA at least), so small batches share the GPU instead of each
        // filling it; and a launch with more tasks than the GPU has CTA
        // slots takes three quarters of them, so the launches queued behind
        // it start on the rest instead of waiting for it to drain (p99 at
        // 20,000 requests/s 2.6-3.2 ms instead of 3.2-10 ms).
        // Requests carry uniform or alpha weights: the byte-row kernel.
        const uint32_t cap = total > (uint32_t)S->grid ? (uint32_t)S->grid * 3 / 4 : (uint32_t)S->grid;
        e = launch_encode_batch(S->G, slot.d_images, nullptr, slot.d_start, n, (int)total, slot.d_counter,
                                slot.stream, (int)std::min<uint32_t>(cap, (total + 3) / 4), nullptr, nullptr, true,
                                listed_tasks ? lists : BatchLists{nullptr, nullptr, nullptr});
    }
    for (size_t i = 0; i < reqs.size() && e == cudaSuccess; i++) {
        Request *q = reqs[i];
        const ImageDesc &d = slot.h_images[i];
        e = cudaMemcpyAsync(S->h_stage + q->host_off, d.out, (size_t)d.nblocks * 8, cudaMemcpyDeviceToHost,
                            slot.stream);
        if (e == cudaSuccess && q->r.errors)
            e = cudaMemcpyAsync(S->h_stage + q->host_off + round_up((size_t)d.nblocks * 8, kGranule), d.errors,
                                (size_t)d.nblocks * 4, cudaMemcpyDeviceToHost, slot.stream);
    }
    if (e == cudaSuccess) e = cudaLaunchHostFunc(slot.stream, on_slot_done, &slot);
    if (e != cudaSuccess) {
        // Nothing was queued behind the failure: finish the slot right away.
        cudaStreamSynchronize(slot.stream);
        slot.status = e == cudaErrorMemoryAllocation ? ICBC_GPU_ERR_OUT_OF_MEMORY : ICBC_GPU_ERR_CUDA;
        slot.done.store(true, std::memory_order_release);
    }
    return slot.status;
}

// Frees the slots whose launches finished and their requests' device and
// input staging space (the GPU is done with them), and queues the requests
// for delivery.  Lock held.
void reap(icbc_gpu_server *S) {
    for (Slot &slot : S->slots) {
        if (!slot.busy || !slot.done.load(std::memory_order_acquire)) continue;
        std::vector<Request *> reqs;
        reqs.swap(slot.reqs);
        for (Request *q : reqs) {
            S->dev.release(q->dev_off, q->dev_bytes);
            if (q->staged) S->in.release(q->in_off, q->in_bytes);
        }
        S->delivery.emplace_back(std::move(reqs), slot.status);
        slot.busy = false;
        slot.status = ICBC_GPU_OK;
        slot.done.store(false, std::memory_order_relaxed);
        S->in_flight--;
        S->cv_deliver.notify_one();
    }
}

// The delivery thread: copies each finished request's blocks (and errors)
// from pinned staging to the caller's buffers, then frees the staging and
// records the request as done.  Runs until the scheduler has stopped and
// everything is delivered.
void deliver(icbc_gpu_server *S) {
    std::unique_lock<std::mutex> lock(S->m);
    for (;;) {
        if (S->delivery.empty()) {
            if (S->scheduler_done) break;
            S->cv_deliver.wait(lock);
            continue;
        }
        std::vector<Request *> reqs = std::move(S->delivery.front().first);
        const int status = S->delivery.front().second;
        S->delivery.pop_front();
        lock.unlock();
        if (status == ICBC_GPU_OK) {
            for (Request *q : reqs) {
                const size_t nb = (size_t)q->d.nblocks;
                std::memcpy(q->r.out, S->h_stage + q->host_off, nb * 8);
                if (q->r.errors)
                    std::memcpy(q->r.errors, S->h_stage + q->host_off + round_up(nb * 8, kGranule), nb * 4);
            }
        }
        const double t = now_ms();
        lock.lock();
        for (Request *q : reqs) {
            S->host.release(q->host_off, q->host_bytes);
            S->live.erase(q->id);
            S->finished[q->id] = status;
            if (status == ICBC_GPU_OK) {
                S->completed++;
                S->latencies.push_back(t - q->t_submit);
                S->pixels += (double)q->r.width * q->r.height;
            } else {
                S->failed++;
            }
            delete q;
        }
        S->cv_done.notify_all();
        S->cv_work.notify_one();  // staging space freed: admission may go on
    }
}

void scheduler(icbc_gpu_server *S) {
    cudaSetDevice(S->device);
    std::unique_lock<std::mutex> lock(S->m);
    for (;;) {
        reap(S);
        // Admission, first come first served: stop at the first request that
        // does not fit, so a large one is not starved by small ones.
        while (!S->pending.empty()) {
            Request *q = S->pending.front();
            size_t doff = 0, hoff = 0;
            if (!S->dev.alloc(q->dev_bytes, &doff)) break;
            if (!S->host.alloc(q->host_bytes, &hoff)) {
                S->dev.release(doff, q->dev_bytes);
                break;
            }
            q->dev_off = doff;
            q->host_off = hoff;
            S->pending.pop_front();
            S->admitted.push_back(q);
            S->arena_peak = std::max<int64_t>(S->arena_peak, (int64_t)S->dev.used());
        }
        // Launch the admitted requests on a free slot: the light ones
        // together or the heavy ones together -- the light ones when only
        // they wait, and when both wait, light and heavy in turn (so heavy
        // requests are not held back for good under a stream of light ones).
        Slot *free_slot = nullptr;
        for (Slot &slot : S->slots)
            if (!slot.busy) { free_slot = &slot; break; }
        if (free_slot && !S->admitted.empty()) {
            const bool any_light =
                std::any_of(S->admitted.begin(), S->admitted.end(), [](const Request *q) { return !q->heavy; });
            const bool any_heavy =
                std::any_of(S->admitted.begin(), S->admitted.end(), [](const Request *q) { return q->heavy; });
            const bool light = any_light && !(any_heavy && S->heavy_turn);
            if (any_light && any_heavy) S->heavy_turn = !S->heavy_turn;
            std::vector<Request *> &take = free_slot->reqs;
            take.clear();
            std::deque<Request *> rest;
            for (Request *q : S->admitted) {
                if (q->heavy != light && take.size() < (size_t)S->cfg.max_batch_images) take.push_back(q);
                else rest.push_back(q);
            }
            S->admitted.swap(rest);
            free_slot->busy = true;
            S->in_flight++;
            S->batches++;
            lock.unlock();
            launch_slot(S, *free_slot);
            lock.lock();
            continue;
        }
        if (S->stop && S->admitted.empty() && S->in_flight == 0) break;
        S->cv_work.wait_for(lock, std::chrono::microseconds(100));
    }
    S->scheduler_done = true;
    S->cv_deliver.notify_all();
}

}  // namespace

extern "C" {

int icbc_gpu_server_create(const icbc_gpu_server_config *config, icbc_gpu_server **server) {
    if (!config || !server || config->hbm_budget_bytes <= 0 || config->max_inflight < 1 || config->max_inflight > 8 ||
        config->max_batch_images < 1 || config->max_batch_images > 4096)
        return ICBC_GPU_ERR_INVALID_ARGUMENT;
    *server = nullptr;
    const GlobalTables *G = nullptr;
    int st = ensure_tables_on_device(&G);
    if (st) return st;
    icbc_gpu_server *S = new icbc_gpu_server();
    S->cfg = *config;
    S->G = G;
    cudaGetDevice(&S->device);
    int per_sm = 1;
    cudaDeviceGetAttribute(&S->grid, cudaDevAttrMultiProcessorCount, S->device);
    // Both queries load the server's kernels now (modules load on first
    // use), not inside the first launches.
    per_sm = batch_ctas_per_sm(true);
    prepare_batch_trivial();
    S->grid *= per_sm;
    const size_t budget = round_up((size_t)config->hbm_budget_bytes, kGranule);
    // Pinned staging for blocks and errors (an eighth and a sixteenth of the
    // texel bytes), capped at 1 GiB: when full, admission waits for space
    // like it does for the device arena.
    const size_t stage = round_up(std::min<size_t>(budget / 4 + (16 << 20), (size_t)1 << 30), kGranule);
    // Pinned input staging: submit() copies texels here so the scheduler only
    // issues DMA; when it is full a request is copied from its pageable
    // buffer at launch instead.
    const size_t in_stage = round_up(std::min<size_t>(budget, (size_t)2 << 30), kGranule);
    cudaError_t e = cudaMalloc(&S->d_arena, budget);
    if (e == cudaSuccess) e = cudaMallocHost(&S->h_stage, stage);
    if (e == cudaSuccess) e = cudaMallocHost(&S->h_in, in_stage);
    S->slots = std::vector<Slot>((size_t)config->max_inflight);
    const size_t n = (size_t)config->max_batch_images;
    for (Slot &slot : S->slots) {
        slot.wake = &S->cv_work;
        if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&slot.stream, cudaStreamNonBlocking);
        if (e == cudaSuccess) e = cudaMalloc(&slot.d_images, sizeof(ImageDesc) * n);
        if (e == cudaSuccess) e = cudaMalloc(&slot.d_start, sizeof(uint32_t) * (n + 1));
        if (e == cudaSuccess) e = cudaMalloc(&slot.d_counter, sizeof(int));
        if (e == cudaSuccess) e = cudaMallocHost(&slot.h_images, sizeof(ImageDesc) * n);
        if (e == cudaSuccess) e = cudaMallocHost(&slot.h_start, sizeof(uint32_t) * (n + 1));
        if (e == cudaSuccess) e = cudaMalloc(&slot.d_list_base, sizeof(int64_t) * n);
        if (e == cudaSuccess) e = cudaMalloc(&slot.d_listed, sizeof(unsigned int) * n);
        if (e == cudaSuccess) e = cudaMallocHost(&slot.h_list_base, sizeof(int64_t) * n);
    }
    if (e != cudaSuccess) {
        icbc_gpu_server_destroy(S);
        return e == cudaErrorMemoryAllocation ? ICBC_GPU_ERR_OUT_OF_MEMORY : ICBC_GPU_ERR_CUDA;
    }
    S->dev.reset(budget);
    S->host.reset(stage);
    S->in.reset(in_stage);
    S->worker = std::thread(scheduler, S);
    S->deliverer = std::thread(deliver, S);
    *server = S;
    return ICBC_GPU_OK;
}

int icbc_gpu_server_submit(icbc_gpu_server *S, const icbc_gpu_request *req, uint64_t *id) {
    if (!S || !req || !id) return ICBC_GPU_ERR_INVALID_ARGUMENT;
    if (!req->rgba || !req->out || req->width < 1 || req->height < 1 || req->pitch < 4 * (int64_t)req->width ||
        req->weight_mode < 0 || req->weight_mode > 1 || req->level < 0 || req->level > 9)
        return ICBC_GPU_ERR_INVALID_ARGUMENT;
    Request *q = new Request();
    q->r = *req;
    // Resolve (level, decoder, flags, weights) as the plain form does, with a
    // placeholder device address; the arena address is filled at launch.
    icbc_gpu_image im;
    std::memset(&im, 0, sizeof(im));
    im.rgba = reinterpret_cast<const uint8_t *>((uintptr_t)256);
    im.width = req->width;
    im.height = req->height;
    im.pitch = (int64_t)round_up(4 * (size_t)req->width, 16);
    im.weight_mode = req->weight_mode;
    im.level = req->level;
    im.decoder = req->decoder;
    im.three_color_mode = req->three_color_mode;
    im.three_color_black = req->three_color_black;
    std::memcpy(im.color_weights, req->color_weights, sizeof(im.color_weights));
    im.out = reinterpret_cast<void *>((uintptr_t)256);
    int st = resolve_image_desc_checked(im, q->d);
    if (st) {
        delete q;
        return st;
    }
    size_request(S, q);
    q->heavy = heavy_request(q->d);
    const size_t img = round_up((size_t)q->dpitch * req->height, kGranule);
    q->out_off = img;
    q->err_off = img + round_up((size_t)q->d.nblocks * 8, kGranule);
    std::unique_lock<std::mutex> lock(S->m);
    if (round_up(q->dev_bytes, kGranule) > S->dev.size() || round_up(q->host_bytes, kGranule) > S->host.size()) {
        S->rejected++;
        delete q;
        return ICBC_GPU_ERR_BUDGET;
    }
    if (S->stop) {
        delete q;
        return ICBC_GPU_ERR_CANCELLED;
    }
    // Levels 4-9 start from zero blocks (the kernels keep prior bytes where
    // no candidate is finite): staged, they travel with the texels in one
    // copy; otherwise the launch clears them.
    const size_t zero_blocks = req->level >= 4 ? (size_t)q->d.nblocks * 8 : 0;
    q->in_bytes = zero_blocks ? q->out_off + zero_blocks : (size_t)q->dpitch * req->height;
    q->staged = S->in.alloc(q->in_bytes, &q->in_off);
    if (q->staged) {
        // The region belongs to this request now: fill it without the lock.
        lock.unlock();
        const size_t row = 4 * (size_t)req->width;
        for (int32_t y = 0; y < req->height; y++)
            std::memcpy(S->h_in + q->in_off + (size_t)y * q->dpitch, req->rgba + (size_t)y * req->pitch, row);
        if (zero_blocks) std::memset(S->h_in + q->in_off + q->out_off, 0, zero_blocks);
        lock.lock();
    }
    q->id = S->next_id++;
    q->t_submit = now_ms();
    S->pending.push_back(q);
    S->live[q->id] = q;
    S->submitted++;
    *id = q->id;
    S->cv_work.notify_one();
    return ICBC_GPU_OK;
}

int icbc_gpu_server_poll(icbc_gpu_server *S, uint64_t id) {
    if (!S) return ICBC_GPU_ERR_INVALID_ARGUMENT;
    std::lock_guard<std::mutex> lock(S->m);
    auto f = S->finished.find(id);
    if (f != S->finished.end()) return f->second;
    return S->live.count(id) ? ICBC_GPU_ERR_NOT_READY : ICBC_GPU_ERR_NOT_FOUND;
}

int icbc_gpu_server_wait(icbc_gpu_server *S, uint64_t id, int32_t timeout_ms) {
    if (!S) return ICBC_GPU_ERR_INVALID_ARGUMENT;
    std::unique_lock<std::mutex> lock(S->m);
    auto ready = [&] { return S->finished.count(id) || !S->live.count(id); };
    if (timeout_ms < 0) S->cv_done.wait(lock, ready);
    else S->cv_done.wait_for(lock, std::chrono::milliseconds(timeout_ms), ready);
    auto f = S->finished.find(id);
    if (f != S->finished.end()) return f->second;
    return S->live.count(id) ? ICBC_GPU_ERR_NOT_READY : ICBC_GPU_ERR_NOT_FOUND;
}

int icbc_gpu_server_cancel(icbc_gpu_server *S, uint64_t id) {
    if (!S) return ICBC_GPU_ERR_INVALID_ARGUMENT;
    std::lock_guard<std::mutex> lock(S->m);
    for (auto it = S->pending.begin(); it != S->pending.end(); ++it) {
        if ((*it)->id == id) {
            Request *q = *it;
            S->pending.erase(it);
            if (q->staged) S->in.release(q->in_off, q->in_bytes);
            S->live.erase(id);
            S->finished[id] = ICBC_GPU_ERR_CANCELLED;
            S->cancelled++;
            delete q;
            S->cv_done.notify_all();
            return ICBC_GPU_OK;
        }
    }
    auto f = S->finished.find(id);
    if (f != S->finished.end()) return f->second == ICBC_GPU_ERR_CANCELLED ? ICBC_GPU_OK : ICBC_GPU_ERR_NOT_READY;
    return S->live.count(id) ? ICBC_GPU_ERR_NOT_READY : ICBC_GPU_ERR_NOT_FOUND;
}

int icbc_gpu_server_get_stats(icbc_gpu_server *S, icbc_gpu_server_stats *out) {
    if (!S || !out) return ICBC_GPU_ERR_INVALID_ARGUMENT;
    std::vector<double> lat;
    {
        std::lock_guard<std::mutex> lock(S->m);
        std::memset(out, 0, sizeof(*out));
        out->submitted = S->submitted;
        out->completed = S->completed;
        out->rejected = S->rejected;
        out->cancelled = S->cancelled;
        out->failed = S->failed;
        out->pending = (int64_t)(S->pending.size() + S->admitted.size());
        out->in_flight = S->in_flight;
        out->batches = S->batches;
        out->arena_bytes = (int64_t)S->dev.size();
        out->arena_used = (int64_t)S->dev.used();
        out->arena_peak = S->arena_peak;
        out->pixels_completed = S->pixels;
        lat = S->latencies;
    }
    if (!lat.empty()) {
        std::sort(lat.begin(), lat.end());
        double sum = 0.0;
        for (double v : lat) sum += v;
        out->latency_mean_ms = sum / lat.size();
        out->latency_p50_ms = lat[(lat.size() - 1) / 2];
        out->latency_p99_ms = lat[std::min(lat.size() - 1, (size_t)((lat.size() - 1) * 0.99 + 0.5))];
        out->latency_max_ms = lat.back();
    }
    return ICBC_GPU_OK;
}

int icbc_gpu_server_destroy(icbc_gpu_server *S) {
    if (!S) return ICBC_GPU_OK;
    {
        std::lock_guard<std::mutex> lock(S->m);
        S->stop = true;
        for (Request *q : S->pending) {
            S->live.erase(q->id);
            S->finished[q->id] = ICBC_GPU_ERR_CANCELLED;
            S->cancelled++;
            delete q;
        }
        S->pending.clear();
        S->cv_work.notify_all();
    }
    if (S->worker.joinable()) S->worker.join();
    if (S->deliverer.joinable()) S->deliverer.join();
    for (Slot &slot : S->slots) {
        if (slot.stream) cudaStreamSynchronize(slot.stream);
        if (slot.stream) cudaStreamDestroy(slot.stream);
        if (slot.d_images) cudaFree(slot.d_images);
        if (slot.d_start) cudaFree(slot.d_start);
        if (slot.d_counter) cudaFree(slot.d_counter);
        if (slot.h_images) cudaFreeHost(slot.h_images);
        if (slot.h_start) cudaFreeHost(slot.h_start);
        if (slot.d_list_base) cudaFree(slot.d_list_base);
        if (slot.d_listed) cudaFree(slot.d_listed);
        if (slot.h_list_base) cudaFreeHost(slot.h_list_base);
    }
    if (S->d_arena) cudaFree(S->d_arena);
    if (S->h_stage) cudaFreeHost(S->h_stage);
    if (S->h_in) cudaFreeHost(S->h_in);
    {
        std::lock_guard<std::mutex> lock(S->m);
        S->cv_done.notify_all();
    }
    delete S;
    return ICBC_GPU_OK;
}

}  // extern "C"
