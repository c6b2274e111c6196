// server.cpp — continuous-batching render server over the batch C ABI.
//
// Requests are queued by client threads; one scheduler thread owns every
// device object.  It keeps up to `slots` batches in flight, each on its own
// non-blocking stream.  When a slot is free it takes the oldest waiting
// requests, uploads them as one batch, sizes the frame with the sizing
// network (sr_batch_plan) and enqueues it (sr_batch_enqueue) without
// waiting, so the next batch is assembled and uploaded while earlier ones
// render.  Finished images are copied into per-request device buffers from
// a stream-ordered pool, and the slot is reused at once.  Admission keeps
// the bytes of the batches in flight plus the uncollected images under the
// memory budget, using the predicted sizes.
#include <algorithm>
#include <cmath>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <mutex>
#include <string>
#include <thread>
#include <unordered_map>
#include <vector>

#include <cuda_runtime.h>

#include "../../include/sr.h"

namespace {

// Batches of at most this many paths are sized by their paths' allotments.
constexpr size_t kSmallBatchPaths = 8192;

struct Request {
    uint64_t id = 0;
    uint32_t W = 0, H = 0;
    std::vector<float> pos;
    std::vector<uint32_t> pos_path, curve_pos, curve_type, curve_path, fill_rule, fill_info;
    float mvp[16];
    double t_submit = 0, t_admit = 0, t_done = 0;
    uint64_t predicted_bytes = 0;
    uint32_t batch_scenes = 0, refit = 0;
    sr_status status = SR_OK;
    void* d_image = nullptr;
    bool done = false;

    size_t image_bytes() const { return (size_t)W * H * 4; }
    sr_scene_view view() const {
        sr_scene_view v{};
        v.n_points = (uint32_t)pos_path.size();
        v.n_curves = (uint32_t)curve_type.size();
        v.n_paths = (uint32_t)fill_rule.size();
        v.position = pos.data();
        v.pos_path_idx = pos_path.data();
        v.curve_pos_map = curve_pos.data();
        v.curve_type = curve_type.data();
        v.curve_path_idx = curve_path.data();
        v.fill_rule = fill_rule.data();
        v.fill_info = fill_info.data();
        return v;
    }
};

struct Slot {
    sr_batch* batch = nullptr;
    cudaStream_t stream = nullptr;
    std::vector<Request*> reqs;
    bool busy = false;
    uint64_t bytes = 0;
};

}  // namespace

namespace sr {
sr_status report_error(sr_status s, const char* msg);   // sets sr_last_error()
}

namespace {

sr_status srv_fail(sr_status s, const char* m) { return sr::report_error(s, m); }

double now_s(std::chrono::steady_clock::time_point t0) {
    return std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
}

}  // namespace

struct sr_server {
    sr_server_opts o{};
    const sr_sizer* sizer = nullptr;
    std::chrono::steady_clock::time_point t0;
    std::mutex mu;
    std::condition_variable cv_work, cv_done;
    std::deque<Request*> pending;
    std::unordered_map<uint64_t, Request*> reqs;
    std::vector<Slot> slots;
    cudaMemPool_t pool = nullptr;
    cudaStream_t copy_stream = nullptr;
    // Images fetched to host memory pass through this pinned buffer: a copy
    // straight into pageable memory went through a slow path whose first
    // use took about 20 ms, and other threads' CUDA calls (the scheduler's)
    // waited behind it.
    std::mutex bounce_mu;
    unsigned char* bounce = nullptr;
    size_t bounce_cap = 0;
    std::thread worker;
    bool stop = false;
    uint64_t next_id = 1;
    uint64_t held = 0;           // bytes of batches in flight + uncollected images
    sr_server_stats st{};
    // admission waits for memory: set when the oldest request does not fit,
    // cleared whenever held bytes drop
    bool budget_blocked = false;

    void run();
    void retire(Slot& sl);
    void hand_over(Slot& sl, sr_status s);
    void grow_idle_slots(const Slot& model);
    bool admit(Slot& sl);
};

extern "C" uint32_t sr_admission_take(const uint64_t* req_bytes, uint32_t n, uint64_t held_bytes, uint64_t budget,
                                      uint32_t max_take, int* rejected) {
    if (rejected) *rejected = 0;
    if (!req_bytes || n == 0 || max_take == 0) return 0;
    if (req_bytes[0] > budget) {
        if (rejected) *rejected = 1;
        return 0;
    }
    uint32_t k = 0;
    uint64_t sum = held_bytes;
    while (k < n && k < max_take && sum + req_bytes[k] <= budget && sum + req_bytes[k] >= sum) {
        sum += req_bytes[k];
        ++k;
    }
    return k;
}

// Waits for the slot's frame (rerun with exact sizing if it overflowed)
// and hands its images over.
void sr_server::retire(Slot& sl) {
    sr_batch_stats b0{}, b1{};
    sr_batch_get_stats(sl.batch, &b0);
    sr_status s = sr_batch_finish(sl.batch);
    sr_batch_get_stats(sl.batch, &b1);
    if (b1.overflows > b0.overflows || b1.refits > b0.refits) {
        std::lock_guard<std::mutex> lk(mu);
        st.overflows += b1.overflows - b0.overflows;
        st.refits += b1.refits - b0.refits;
        for (Request* r : sl.reqs) r->refit = 1;
    }
    hand_over(sl, s);
}

// Copies each request's image out of the slot's batch into a buffer of its
// own (stream-ordered pool), marks the requests done and frees the slot.
void sr_server::hand_over(Slot& sl, sr_status s) {
    uint64_t image_total = 0;
    for (size_t i = 0; i < sl.reqs.size(); ++i) {
        Request* r = sl.reqs[i];
        r->status = s;
        if (s != SR_OK) continue;
        if (cudaMallocFromPoolAsync(&r->d_image, r->image_bytes(), pool, sl.stream) == cudaSuccess) {
            r->status = sr_batch_get_image(sl.batch, (uint32_t)i, r->d_image, 1, sl.stream);
            image_total += r->image_bytes();
        } else {
            r->d_image = nullptr;
            r->status = SR_ERR_OOM;
        }
    }
    cudaStreamSynchronize(sl.stream);
    std::lock_guard<std::mutex> lk(mu);
    const double t = now_s(t0);
    for (Request* r : sl.reqs) {
        r->t_done = t;
        r->done = true;
    }
    held = held - sl.bytes + image_total;
    st.peak_bytes = std::max(st.peak_bytes, held);
    budget_blocked = false;
    st.completed += sl.reqs.size();
    sl.reqs.clear();
    sl.busy = false;
    sl.bytes = 0;
    cv_done.notify_all();
    grow_idle_slots(sl);
}

// A slot's first batch larger than any before reallocates its buffers
// behind a device-wide wait (about 10 ms at serving sizes, which the queue
// behind it pays).  When a slot's buffers have grown, the idle slots grow
// like it at once, so that each size is paid for once, not once per slot.
void sr_server::grow_idle_slots(const Slot& model) {
    uint64_t want = 0;
    if (sr_batch_held_bytes(model.batch, &want) != SR_OK) return;
    for (Slot& other : slots) {
        if (&other == &model || other.busy) continue;
        uint64_t have = 0;
        if (sr_batch_held_bytes(other.batch, &have) != SR_OK || have >= want) continue;
        sr_batch_reserve_like(other.batch, model.batch);   // best effort: a failure only leaves it smaller
    }
}

// Forms, sizes and enqueues one batch in a free slot; false when nothing
// could be admitted now.
bool sr_server::admit(Slot& sl) {
    std::vector<Request*> take;
    {
        std::lock_guard<std::mutex> lk(mu);
        const size_t n = std::min<size_t>(pending.size(), o.max_batch_scenes);
        for (size_t i = 0; i < n; ++i) take.push_back(pending[i]);
    }
    if (take.empty()) return false;
    auto form = [&](size_t count) -> sr_status {
        sr_status s = sr_batch_clear(sl.batch);
        for (size_t i = 0; i < count && s == SR_OK; ++i) {
            sr_scene_view v = take[i]->view();
            s = sr_batch_add_scene(sl.batch, take[i]->W, take[i]->H, &v, take[i]->mvp, nullptr);
        }
        if (s == SR_OK) s = sr_batch_commit(sl.batch);
        return s;
    };
    auto fail_requests = [&](size_t count, sr_status s) {
        std::lock_guard<std::mutex> lk(mu);
        for (size_t i = 0; i < count; ++i) {
            take[i]->status = s;
            take[i]->done = true;
            take[i]->t_done = now_s(t0);
            pending.pop_front();
        }
        st.completed += count;
        cv_done.notify_all();
    };
    sr_status s = form(take.size());
    if (s != SR_OK) {
        fail_requests(take.size(), s);
        return true;
    }
    sr_batch_render_opts ro{};
    ro.struct_size = sizeof ro;
    ro.refit_on_overflow = 1;
    if (sizer) {
        sr_sizing_plan plan{};
        std::vector<int64_t> caps(2 * take.size());
        s = sr_batch_plan(sl.batch, sizer, &o.margins, &plan, caps.data(), sl.stream);
        if (s != SR_OK) {
            fail_requests(take.size(), s);
            return true;
        }
        // The frame margin is calibrated where the errors of many paths
        // average out; a batch of few paths (most batches under a steady
        // request stream) is sized by the sum of its paths' own allotments
        // instead, whose margins make an overflow -- and the whole-batch
        // rerun with exact sizing that follows it -- rare.  Each scene's
        // capacities grow by the batch's factor before admission, so that
        // the requests' shares of the budget cover them.
        {
            size_t paths = 0;
            int64_t rall = 0, dall = 0;
            for (size_t i = 0; i < take.size(); ++i) {
                paths += take[i]->fill_rule.size();
                rall += caps[2 * i];
                dall += caps[2 * i + 1];
            }
            if (paths <= kSmallBatchPaths && (plan.path_records > rall || plan.path_draws > dall)) {
                const double fr = std::max(1.0, (double)plan.path_records / (double)std::max<int64_t>(rall, 1));
                const double fd = std::max(1.0, (double)plan.path_draws / (double)std::max<int64_t>(dall, 1));
                int64_t r2 = 0, d2 = 0;
                for (size_t i = 0; i < take.size(); ++i) {
                    caps[2 * i] = (int64_t)std::ceil((double)caps[2 * i] * fr);
                    caps[2 * i + 1] = (int64_t)std::ceil((double)caps[2 * i + 1] * fd);
                    r2 += caps[2 * i];
                    d2 += caps[2 * i + 1];
                }
                uint64_t fb = 0;
                if (sr_batch_frame_bytes(sl.batch, r2, std::min<int64_t>(std::max<int64_t>(d2, 1), 2 * std::max<int64_t>(r2, 1)),
                                         &fb) == SR_OK)
                    plan.device_bytes = fb;
            }
        }
        // each request's share of the batch bytes, by its predicted records
        // and draw records, plus the copy of its finished image
        double weight = 0;
        for (size_t i = 0; i < take.size(); ++i) weight += (double)caps[2 * i] + (double)caps[2 * i + 1] + 1.0;
        std::vector<uint64_t> share(take.size());
        for (size_t i = 0; i < take.size(); ++i)
            share[i] = (uint64_t)((double)plan.device_bytes * ((double)caps[2 * i] + (double)caps[2 * i + 1] + 1.0) /
                                  weight) +
                       take[i]->image_bytes();
        int rejected = 0;
        uint32_t k;
        {
            std::lock_guard<std::mutex> lk(mu);
            k = sr_admission_take(share.data(), (uint32_t)share.size(), held, o.memory_budget,
                                  (uint32_t)share.size(), &rejected);
        }
        if (rejected) {
            std::lock_guard<std::mutex> lk(mu);
            Request* r = pending.front();
            pending.pop_front();
            r->status = SR_ERR_OOM;
            r->done = true;
            r->t_done = now_s(t0);
            ++st.rejected;
            ++st.completed;
            cv_done.notify_all();
            return true;
        }
        if (k == 0) {
            std::lock_guard<std::mutex> lk(mu);
            ++st.budget_waits;
            budget_blocked = true;
            return false;
        }
        // capacities of the admitted scenes (grown by the batch factor above)
        int64_t rec = 0, drw = 0;
        uint64_t bytes = 0;
        for (uint32_t i = 0; i < k; ++i) {
            rec += caps[2 * i];
            drw += caps[2 * i + 1];
            bytes += share[i];
        }
        if (k < take.size()) {
            ++st.budget_waits;
            take.resize(k);
            s = form(k);
            if (s != SR_OK) {
                fail_requests(k, s);
                return true;
            }
        }
        ro.record_capacity = rec;
        ro.draw_capacity = std::min<int64_t>(std::max<int64_t>(drw, 1), 2 * std::max<int64_t>(rec, 1));
        {
            std::lock_guard<std::mutex> lk(mu);
            for (uint32_t i = 0; i < k; ++i) {
                pending.pop_front();
                take[i]->predicted_bytes = share[i];
                take[i]->batch_scenes = k;
                take[i]->t_admit = now_s(t0);
            }
            held += bytes;
            st.peak_bytes = std::max(st.peak_bytes, held);
            ++st.batches;
        }
        sl.reqs = take;
        sl.bytes = bytes;
        sl.busy = true;
        s = sr_batch_enqueue(sl.batch, &ro, sl.stream);
        if (s != SR_OK) {
            std::lock_guard<std::mutex> lk(mu);
            for (Request* r : take) {
                r->status = s;
                r->done = true;
                r->t_done = now_s(t0);
            }
            held -= bytes;
            st.completed += take.size();
            sl.reqs.clear();
            sl.busy = false;
            cv_done.notify_all();
        }
        return true;
    }
    // exact sizing: the scheduler waits for the batch's count
    {
        std::lock_guard<std::mutex> lk(mu);
        for (Request* r : take) {
            pending.pop_front();
            r->batch_scenes = (uint32_t)take.size();
            r->t_admit = now_s(t0);
        }
        ++st.batches;
    }
    sl.reqs = take;
    sl.busy = true;
    sl.bytes = 0;
    ro.record_capacity = -1;
    hand_over(sl, sr_batch_render(sl.batch, &ro, sl.stream));
    return true;
}

void sr_server::run() {
    cudaSetDevice(o.device);
    for (;;) {
        bool any_busy = false;
        for (Slot& sl : slots) {
            if (!sl.busy) continue;
            int done = 0;
            if (sr_batch_query(sl.batch, &done) != SR_OK) done = 1;   // finish reports the error
            if (done) {
                retire(sl);
            } else {
                any_busy = true;
            }
        }
        bool admitted = false;
        for (Slot& sl : slots) {
            if (sl.busy) continue;
            bool has_pending;
            {
                std::lock_guard<std::mutex> lk(mu);
                has_pending = !pending.empty() && !budget_blocked;
            }
            if (!has_pending) break;
            if (admit(sl)) admitted = true;
            else break;
        }
        for (const Slot& sl : slots) any_busy = any_busy || sl.busy;
        std::unique_lock<std::mutex> lk(mu);
        if (stop && !any_busy && (pending.empty() || budget_blocked)) {
            // requests that can no longer be admitted end with an error
            for (Request* r : pending) {
                r->status = SR_ERR_INVALID_ARG;
                r->done = true;
                r->t_done = now_s(t0);
            }
            pending.clear();
            cv_done.notify_all();
            return;
        }
        if (admitted) continue;
        if (any_busy) cv_work.wait_for(lk, std::chrono::microseconds(50));
        else cv_work.wait(lk, [&] { return stop || (!pending.empty() && !budget_blocked); });
    }
}

extern "C" {

sr_status sr_server_create(const sr_server_opts* opts, const sr_sizer* sizer, sr_server** out) {
    if (!out) return srv_fail(SR_ERR_INVALID_ARG, "out is NULL");
    *out = nullptr;
    sr_server_opts o{};
    o.struct_size = sizeof o;
    o.mode = SR_MODE_PIXEL;
    o.slots = 2;
    o.max_batch_scenes = 64;
    o.memory_budget = 120ull * 1000 * 1000 * 1000;
    o.margins.struct_size = sizeof(sr_sizing_margins);
    if (opts) {
        if (opts->struct_size < sizeof o) return srv_fail(SR_ERR_INVALID_ARG, "opts.struct_size too small");
        o = *opts;
        o.margins.struct_size = sizeof(sr_sizing_margins);
    }
    if (o.slots == 0 || o.slots > 16 || o.max_batch_scenes == 0 || o.memory_budget == 0)
        return srv_fail(SR_ERR_INVALID_ARG, "slots 1..16, max_batch_scenes and memory_budget > 0");
    if (cudaSetDevice(o.device) != cudaSuccess) return srv_fail(SR_ERR_INVALID_ARG, "device not present");
    sr_server* s = new sr_server();
    s->o = o;
    s->sizer = sizer;
    s->t0 = std::chrono::steady_clock::now();
    cudaMemPoolProps pp{};
    pp.allocType = cudaMemAllocationTypePinned;
    pp.location.type = cudaMemLocationTypeDevice;
    pp.location.id = o.device;
    sr_status status = SR_OK;
    if (cudaMemPoolCreate(&s->pool, &pp) != cudaSuccess) status = SR_ERR_CUDA;
    if (status == SR_OK) {
        uint64_t keep = ~0ull;   // keep freed blocks for reuse
        cudaMemPoolSetAttribute(s->pool, cudaMemPoolAttrReleaseThreshold, &keep);
        if (cudaStreamCreateWithFlags(&s->copy_stream, cudaStreamNonBlocking) != cudaSuccess) status = SR_ERR_CUDA;
    }
    sr_options bo{sizeof(sr_options), o.mode, o.device, 0};
    for (uint32_t i = 0; i < o.slots && status == SR_OK; ++i) {
        Slot sl;
        status = sr_batch_create(&bo, &sl.batch);
        if (status == SR_OK && cudaStreamCreateWithFlags(&sl.stream, cudaStreamNonBlocking) != cudaSuccess)
            status = SR_ERR_CUDA;
        s->slots.push_back(sl);
    }
    if (status != SR_OK) {
        for (Slot& sl : s->slots) {
            if (sl.batch) sr_batch_destroy(sl.batch);
            if (sl.stream) cudaStreamDestroy(sl.stream);
        }
        if (s->copy_stream) cudaStreamDestroy(s->copy_stream);
        if (s->pool) cudaMemPoolDestroy(s->pool);
        delete s;
        return status;
    }
    s->worker = std::thread([s] { s->run(); });
    *out = s;
    return SR_OK;
}

sr_status sr_server_submit(sr_server* s, uint32_t width, uint32_t height, const sr_scene_view* v, const float* mvp,
                           uint64_t* ticket) {
    if (!s || !v || !ticket) return srv_fail(SR_ERR_INVALID_ARG, "NULL argument");
    if (width == 0 || height == 0 || width > 16384 || height > 16384)
        return srv_fail(SR_ERR_INVALID_ARG, "canvas outside 1..16384");
    if ((v->n_points && (!v->position || !v->pos_path_idx)) ||
        (v->n_curves && (!v->curve_pos_map || !v->curve_type || !v->curve_path_idx)) ||
        (v->n_paths && (!v->fill_rule || !v->fill_info)))
        return srv_fail(SR_ERR_INVALID_ARG, "scene array missing");
    Request* r = new Request();
    r->W = width;
    r->H = height;
    r->pos.assign(v->position, v->position + 2 * (size_t)v->n_points);
    r->pos_path.assign(v->pos_path_idx, v->pos_path_idx + v->n_points);
    r->curve_pos.assign(v->curve_pos_map, v->curve_pos_map + v->n_curves);
    r->curve_type.assign(v->curve_type, v->curve_type + v->n_curves);
    r->curve_path.assign(v->curve_path_idx, v->curve_path_idx + v->n_curves);
    r->fill_rule.assign(v->fill_rule, v->fill_rule + v->n_paths);
    r->fill_info.assign(v->fill_info, v->fill_info + v->n_paths);
    static const float kId[16] = {1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1};
    std::memcpy(r->mvp, mvp ? mvp : kId, sizeof r->mvp);
    {
        std::lock_guard<std::mutex> lk(s->mu);
        if (s->stop) {
            delete r;
            return srv_fail(SR_ERR_INVALID_ARG, "server is stopping");
        }
        r->id = s->next_id++;
        r->t_submit = now_s(s->t0);
        s->reqs[r->id] = r;
        s->pending.push_back(r);
        ++s->st.submitted;
        *ticket = r->id;
    }
    s->cv_work.notify_one();
    return SR_OK;
}

sr_status sr_server_wait(sr_server* s, uint64_t ticket, void* rgba_out, int out_is_device, sr_request_info* info,
                         int64_t timeout_ms) {
    if (!s) return srv_fail(SR_ERR_INVALID_ARG, "NULL server");
    Request* r = nullptr;
    {
        std::unique_lock<std::mutex> lk(s->mu);
        auto it = s->reqs.find(ticket);
        if (it == s->reqs.end()) return srv_fail(SR_ERR_INVALID_ARG, "unknown ticket");
        r = it->second;
        auto ready = [&] { return r->done; };
        if (timeout_ms < 0) s->cv_done.wait(lk, ready);
        else if (!s->cv_done.wait_for(lk, std::chrono::milliseconds(timeout_ms), ready))
            return srv_fail(SR_ERR_TIMEOUT, "request not finished");
        s->reqs.erase(it);
    }
    sr_status status = r->status;
    if (r->d_image) {
        cudaSetDevice(s->o.device);
        if (rgba_out && status == SR_OK) {
            const size_t bytes = r->image_bytes();
            cudaError_t e = cudaSuccess;
            if (out_is_device) {
                e = cudaMemcpyAsync(rgba_out, r->d_image, bytes, cudaMemcpyDeviceToDevice, s->copy_stream);
                if (e == cudaSuccess) e = cudaStreamSynchronize(s->copy_stream);
            } else {
                std::lock_guard<std::mutex> bl(s->bounce_mu);
                if (s->bounce_cap < bytes) {
                    if (s->bounce) cudaFreeHost(s->bounce);
                    s->bounce = nullptr;
                    s->bounce_cap = 0;
                    e = cudaMallocHost(&s->bounce, bytes + bytes / 2);
                    if (e == cudaSuccess) s->bounce_cap = bytes + bytes / 2;
                }
                if (e == cudaSuccess)
                    e = cudaMemcpyAsync(s->bounce, r->d_image, bytes, cudaMemcpyDeviceToHost, s->copy_stream);
                if (e == cudaSuccess) e = cudaStreamSynchronize(s->copy_stream);
                if (e == cudaSuccess) std::memcpy(rgba_out, s->bounce, bytes);
            }
            if (e != cudaSuccess) status = srv_fail(SR_ERR_CUDA, cudaGetErrorString(e));
        }
        cudaFreeAsync(r->d_image, s->copy_stream);
        std::lock_guard<std::mutex> lk(s->mu);
        s->held -= r->image_bytes();
        s->budget_blocked = false;
    }
    if (info) {
        std::memset(info, 0, sizeof *info);
        info->submit_s = r->t_submit;
        info->admit_s = r->t_admit;
        info->done_s = r->t_done;
        info->predicted_bytes = r->predicted_bytes;
        info->batch_scenes = r->batch_scenes;
        info->refit = r->refit;
        info->status = r->status;
    }
    delete r;
    s->cv_work.notify_one();   // freed memory may admit more
    if (status != SR_OK && status != SR_ERR_CUDA) srv_fail(status, "request failed");
    return status;
}

sr_status sr_server_get_stats(sr_server* s, sr_server_stats* out) {
    if (!s || !out) return srv_fail(SR_ERR_INVALID_ARG, "NULL argument");
    std::lock_guard<std::mutex> lk(s->mu);
    *out = s->st;
    return SR_OK;
}

void sr_server_destroy(sr_server* s) {
    if (!s) return;
    {
        std::lock_guard<std::mutex> lk(s->mu);
        s->stop = true;
    }
    s->cv_work.notify_all();
    if (s->worker.joinable()) s->worker.join();
    cudaSetDevice(s->o.device);
    for (auto& kv : s->reqs) {
        if (kv.second->d_image) cudaFreeAsync(kv.second->d_image, s->copy_stream);
        delete kv.second;
    }
    cudaStreamSynchronize(s->copy_stream);
    for (Slot& sl : s->slots) {
        sr_batch_destroy(sl.batch);
        cudaStreamDestroy(sl.stream);
    }
    cudaStreamDestroy(s->copy_stream);
    cudaMemPoolDestroy(s->pool);
    if (s->bounce) cudaFreeHost(s->bounce);
    delete s;
}

}  // extern "C"
