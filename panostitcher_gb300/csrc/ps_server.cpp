// ps_server.cpp -- live-stream serving with continuous batching.
//
// The reference serves one rig per task thread and drops frames through a
// real-time queue (source/Task/ConcurrentQueue.h:79-145,
// source/Task/PanoramaLiveStreamTask2.cpp:919-1148).  Here many streams
// share one GPU: each stream's rig (maps, weights, pyramids) stays resident;
// admission checks a device-memory budget like the reference's free-memory
// check (source/Task/RicohUtil.cpp:1135-1170); a scheduler forms a batch per
// tick from the head frame of every idle stream with a frame waiting and runs
// it as one launch sequence.  Two ticks can be in flight on two CUDA
// streams, so frames that arrive while a tick runs are uploaded and launched
// as soon as a slot frees up, overlapping the running tick.
#include <algorithm>
#include <chrono>
#include <deque>
#include <map>
#include <memory>
#include <thread>

#include "ps_rig.h"

using ps::fail;

struct ps_server {
    long long budget = 0;
    int maxBatch = 1;
    std::map<int, std::unique_ptr<ps::Rig>> streams;
    int nextId = 0;
    static constexpr int kSlots = 2;
    static constexpr long long kTickBytes = 256LL << 20;  // host-frame bytes a tick uploads at most
    // a stream has at most one frame in flight, so its rig keeps one state slot
    static constexpr int kRigSlots = 1;
    cudaStream_t cs[kSlots] = {};
    cudaEvent_t end[kSlots] = {};
    ps::Plan plans[kSlots];

    long long resident() const
    {
        long long b = 0;
        for (const auto& kv : streams) b += kv.second->residentBytes();
        return b;
    }
    ~ps_server()
    {
        for (int s = 0; s < kSlots; s++) {
            if (cs[s]) {
                cudaStreamSynchronize(cs[s]);
                cudaStreamDestroy(cs[s]);
            }
            if (end[s]) cudaEventDestroy(end[s]);
        }
    }
};

namespace {
thread_local std::string t_serr;

template <class F>
int sguard(F&& f)
{
    try {
        f();
        return PS_OK;
    } catch (const ps::Error& e) {
        t_serr = e.what();
        return e.code;
    } catch (const std::bad_alloc&) {
        t_serr = "host allocation failed";
        return PS_ENOMEM;
    } catch (const std::exception& e) {
        t_serr = e.what();
        return PS_EINVAL;
    }
}
}  // namespace

// server errors are reported through the same ps_last_error() text
static int forward(int st)
{
    if (st != PS_OK) ps::setLastError(t_serr);
    return st;
}

extern "C" {

int ps_server_create(long long budget_bytes, int max_batch, ps_server** out)
{
    return forward(sguard([&] {
        if (!out) fail(PS_EINVAL, "out is NULL");
        if (budget_bytes <= 0) fail(PS_EINVAL, "budget must be positive");
        if (max_batch <= 0) fail(PS_EINVAL, "max_batch must be positive");
        std::unique_ptr<ps_server> s(new ps_server());
        s->budget = budget_bytes;
        s->maxBatch = max_batch;
        for (int k = 0; k < ps_server::kSlots; k++) {
            PS_CUDA(cudaStreamCreateWithFlags(&s->cs[k], cudaStreamNonBlocking));
            PS_CUDA(cudaEventCreate(&s->end[k]));
        }
        *out = s.release();
    }));
}

void ps_server_destroy(ps_server* s) { delete s; }

int ps_server_admit(ps_server* s, const ps_photo_param* params, int num_params, int blend_param, int src_w,
                    int src_h, int dst_w, int dst_h, int* stream_id)
{
    return forward(sguard([&] {
        if (!s || !stream_id) fail(PS_EINVAL, "NULL argument");
        const long long est = ps::Rig::estimateBytes(params, num_params, blend_param, src_w, src_h, dst_w, dst_h,
                                                     ps_server::kRigSlots);
        const long long used = s->resident();
        if (used + est > s->budget)
            fail(PS_ENOMEM, "stream needs about %lld bytes; %lld of the %lld-byte budget are in use", est, used,
                 s->budget);
        std::unique_ptr<ps::Rig> rig(new ps::Rig());
        rig->setSlots(ps_server::kRigSlots);
        rig->prepareFromParams(params, num_params, blend_param, src_w, src_h, dst_w, dst_h, nullptr,
                               s->cs[0]);
        if (used + rig->residentBytes() > s->budget)
            fail(PS_ENOMEM, "stream holds %lld bytes; %lld of the %lld-byte budget are in use",
                 rig->residentBytes(), used, s->budget);
        *stream_id = s->nextId++;
        s->streams[*stream_id] = std::move(rig);
    }));
}

int ps_server_remove(ps_server* s, int stream_id)
{
    return forward(sguard([&] {
        if (!s) fail(PS_EINVAL, "server is NULL");
        auto it = s->streams.find(stream_id);
        if (it == s->streams.end()) fail(PS_EINVAL, "no stream %d", stream_id);
        for (int k = 0; k < ps_server::kSlots; k++) PS_CUDA(cudaStreamSynchronize(s->cs[k]));
        for (auto& p : s->plans) p.bind({});
        s->streams.erase(it);
    }));
}

long long ps_server_resident_bytes(const ps_server* s) { return s ? s->resident() : 0; }

int ps_server_run_trace(ps_server* s, int num_frames, const int* stream_ids, const long long* arrival_ns,
                        const ps_image* const* srcs, const uint8_t* const* luts, ps_image* dsts,
                        long long* latency_ns, long long* wall_ns)
{
    return forward(sguard([&] {
        if (!s || num_frames <= 0 || !stream_ids || !arrival_ns || !srcs || !latency_ns)
            fail(PS_EINVAL, "bad trace arguments");
        std::map<int, std::deque<int>> pending;
        std::map<int, bool> busy;
        for (int k = 0; k < num_frames; k++) {
            auto it = s->streams.find(stream_ids[k]);
            if (it == s->streams.end()) fail(PS_EINVAL, "frame %d: no stream %d", k, stream_ids[k]);
            if (k && arrival_ns[k] < arrival_ns[k - 1]) fail(PS_EINVAL, "arrivals must be sorted");
            if (!srcs[k]) fail(PS_EINVAL, "frame %d has no sources", k);
            const ps::Rig& rig = *it->second;
            for (int i = 0; i < rig.numImages(); i++) {
                const ps_image& im = srcs[k][i];
                if (!im.data || im.width != rig.srcW() || im.height != rig.srcH() ||
                    (im.format != PS_FMT_BGR32 && im.format != PS_FMT_BGR24) || im.format != srcs[k][0].format ||
                    im.pitch < (long long)im.width * (im.format == PS_FMT_BGR24 ? 3 : 4))
                    fail(PS_EINVAL, "frame %d camera %d: bad source image", k, i);
            }
            if (dsts && (dsts[k].width != rig.width() || dsts[k].height != rig.height() || !dsts[k].data))
                fail(PS_EINVAL, "frame %d: bad destination image", k);
            latency_ns[k] = -1;
        }
        // device-resident outputs when the caller wants none back
        std::map<int, ps_image> devOut;
        for (auto& kv : s->streams)
            devOut[kv.first] = ps_image{kv.second->outputBuffer(), (long long)kv.second->width() * 4,
                                        kv.second->width(), kv.second->height(), PS_FMT_BGR32, PS_MEM_DEVICE};

        cudaEvent_t base;
        PS_CUDA(cudaEventCreate(&base));
        PS_CUDA(cudaEventRecord(base, s->cs[0]));
        PS_CUDA(cudaEventSynchronize(base));
        using clk = std::chrono::steady_clock;
        const auto t0 = clk::now();
        auto nowNs = [&] { return (long long)std::chrono::duration_cast<std::chrono::nanoseconds>(clk::now() - t0).count(); };

        std::vector<int> inflight[ps_server::kSlots];
        bool active[ps_server::kSlots] = {};
        int next = 0, done = 0;
        long long lastProgress = 0, lastDone = 0;
        const long long stallLimit = 120LL * 1000000000LL;  // bounded wait: 120 s without progress
        try {
            while (done < num_frames) {
                bool progressed = false;
                const long long now = nowNs();
                while (next < num_frames && arrival_ns[next] <= now) {
                    pending[stream_ids[next]].push_back(next);
                    next++;
                }
                for (int sl = 0; sl < ps_server::kSlots; sl++) {
                    if (!active[sl]) continue;
                    const cudaError_t q = cudaEventQuery(s->end[sl]);
                    if (q == cudaErrorNotReady) continue;
                    PS_CUDA(q);
                    float ms = 0;
                    PS_CUDA(cudaEventElapsedTime(&ms, base, s->end[sl]));
                    const long long doneNs = (long long)((double)ms * 1e6);
                    for (int k : inflight[sl]) {
                        latency_ns[k] = doneNs - arrival_ns[k];
                        busy[stream_ids[k]] = false;
                        done++;
                    }
                    lastDone = std::max(lastDone, doneNs);
                    inflight[sl].clear();
                    active[sl] = false;
                    progressed = true;
                }
                for (int sl = 0; sl < ps_server::kSlots; sl++) {
                    if (active[sl]) continue;
                    // the head frame of every idle stream, oldest first
                    std::vector<std::pair<long long, int>> heads;
                    for (auto& kv : pending)
                        if (!kv.second.empty() && !busy[kv.first])
                            heads.push_back({arrival_ns[kv.second.front()], kv.first});
                    if (heads.empty()) break;
                    std::sort(heads.begin(), heads.end());
                    if ((int)heads.size() > s->maxBatch) heads.resize(s->maxBatch);
                    // every frame of a tick completes with the tick, so a tick
                    // takes frames (oldest first) only up to kTickBytes of
                    // uploads: a small frame is not held behind many large ones
                    long long bytes = 0;
                    size_t take = 0;
                    for (; take < heads.size(); take++) {
                        const ps::Rig& rg = *s->streams[heads[take].second];
                        const long long b = (long long)rg.numImages() * rg.srcW() * rg.srcH() * 4;
                        if (take > 0 && bytes + b > ps_server::kTickBytes) break;
                        bytes += b;
                    }
                    heads.resize(take);
                    std::vector<ps::Rig*> rigs;
                    std::vector<ps::FrameInput> in;
                    for (auto& h : heads) {
                        const int k = pending[h.second].front();
                        pending[h.second].pop_front();
                        busy[h.second] = true;
                        inflight[sl].push_back(k);
                        rigs.push_back(s->streams[h.second].get());
                        in.push_back({srcs[k], luts ? luts[k] : nullptr, dsts ? &dsts[k] : &devOut[h.second]});
                    }
                    s->plans[sl].bind(rigs);
                    s->plans[sl].run(in, s->cs[sl], false);
                    PS_CUDA(cudaEventRecord(s->end[sl], s->cs[sl]));
                    active[sl] = true;
                    progressed = true;
                }
                if (progressed) {
                    lastProgress = nowNs();
                } else {
                    if (nowNs() - lastProgress > stallLimit) fail(PS_ETIMEOUT, "no progress for 120 s");
                    long long wait = 20000;  // poll every 20 us while ticks run
                    bool anyActive = false;
                    for (int sl = 0; sl < ps_server::kSlots; sl++) anyActive = anyActive || active[sl];
                    if (next < num_frames && !anyActive)
                        wait = std::max(0LL, std::min(arrival_ns[next] - nowNs(), 1000000LL));
                    if (wait > 0) std::this_thread::sleep_for(std::chrono::nanoseconds(wait));
                }
            }
        } catch (...) {
            for (int sl = 0; sl < ps_server::kSlots; sl++) cudaStreamSynchronize(s->cs[sl]);
            cudaEventDestroy(base);
            throw;
        }
        cudaEventDestroy(base);
        if (wall_ns) *wall_ns = lastDone;
    }));
}

}  // extern "C"
