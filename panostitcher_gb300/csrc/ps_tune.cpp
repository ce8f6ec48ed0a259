// ps_tune.cpp -- the launch-shape autotuner.  The reference fixes its
// launch shapes at compile time (CudaAccel's 16x16 blocks); here the
// choices that may change after prepare (LaunchShape) are timed on the
// prepared rig itself, frames issued the way the caller will issue them,
// and the fastest kept.  Every shape computes the same bytes: the tail
// split only moves levels between kernels that run the same per-tile code,
// and grid widths only change which CTA takes which tile.
#include <algorithm>
#include <cstdio>
#include <map>
#include <mutex>
#include <string>
#include <vector>

#include "ps_rig.h"

namespace ps {
namespace {

std::mutex g_tuneMu;
struct Tuned {
    LaunchShape shape;
    TuneReport report;
};
std::map<std::string, Tuned> g_tuned;  // by rig geometry, GPU and concurrency

std::string tuneKey(const Rig& r, int inflight, bool useGraph)
{
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    char head[160];
    std::snprintf(head, sizeof head, "sm%d n%d %dx%d L%d src%dx%d slots%d inflight%d graph%d remap%d", sms,
                  r.numImages(), r.width(), r.height(), r.numLevels(), r.srcW(), r.srcH(), r.slots(), inflight,
                  useGraph ? 1 : 0, r.numRemapItems());
    std::string key = head;
    for (int j = 0; j <= r.numLevels(); j++)
        key += " " + std::to_string(j > 0 ? r.numDownItems(j) : 0) + "/" + std::to_string(r.numBlendItems(j));
    return key;
}

// Frames issued round-robin on `inflight` caller streams, with device
// inputs and one device canvas per stream.  The inputs are the rig's frame
// staging of every state slot, each filled with its own pattern, and frame k
// reads slot k's: with eight slots the trial cycles through more input bytes
// than L2 holds, as a stream of distinct frames does.
class Trials {
public:
    Trials(Rig& rig, Plan& plan, int frames, int inflight, bool useGraph)
        : rig_(rig), plan_(plan), frames_(frames), inflight_(inflight), useGraph_(useGraph)
    {
        const int n = rig.numImages(), W = rig.width(), H = rig.height();
        const long long pitch = rig.inputPitch();
        std::vector<uint8_t> pattern((size_t)pitch * rig.srcH());
        uint32_t x = 0x9E3779B9u;
        src_.resize(rig.slots());
        for (int sl = 0; sl < rig.slots(); sl++) {
            for (uint8_t& b : pattern) {  // xorshift32, continued from slot to slot
                x ^= x << 13;
                x ^= x >> 17;
                x ^= x << 5;
                b = (uint8_t)(x >> 24);
            }
            src_[sl].resize(n);
            for (int c = 0; c < n; c++) {
                PS_CUDA(cudaMemcpy(rig.inputBuffer(c, sl), pattern.data(), pattern.size(), cudaMemcpyHostToDevice));
                src_[sl][c] = {rig.inputBuffer(c, sl), pitch, rig.srcW(), rig.srcH(), PS_FMT_BGR32, PS_MEM_DEVICE};
            }
        }
        luts_.resize((size_t)n * 768);
        for (size_t k = 0; k < luts_.size(); k++) luts_[k] = (uint8_t)std::min<size_t>(255, (k % 256) * 9 / 8);
        out_.resize(inflight);
        dst_.resize(inflight);
        streams_.resize(inflight);
        ends_.resize(inflight);
        for (int s = 0; s < inflight; s++) {
            out_[s].alloc((size_t)W * H * 4);
            dst_[s] = {out_[s].get(), (long long)W * 4, W, H, PS_FMT_BGR32, PS_MEM_DEVICE};
            PS_CUDA(cudaStreamCreateWithFlags(&streams_[s], cudaStreamNonBlocking));
            PS_CUDA(cudaEventCreateWithFlags(&ends_[s], cudaEventDisableTiming));
        }
        PS_CUDA(cudaEventCreate(&t0_));
        PS_CUDA(cudaEventCreate(&t1_));
    }
    ~Trials()
    {
        for (cudaStream_t s : streams_)
            if (s) {
                cudaStreamSynchronize(s);
                cudaStreamDestroy(s);
            }
        for (cudaEvent_t e : ends_)
            if (e) cudaEventDestroy(e);
        if (t0_) cudaEventDestroy(t0_);
        if (t1_) cudaEventDestroy(t1_);
    }

    // ms per frame of a shape: the median of five timed runs (a 1% move must
    // stand out of run-to-run noise of about that size)
    double time(const LaunchShape& shape)
    {
        rig_.setShape(shape);
        plan_.bind({&rig_});
        for (int k = 0; k < 2 * Rig::kIoSlots; k++) issue(k);  // every argument slot captures its graph
        for (cudaStream_t s : streams_) PS_CUDA(cudaStreamSynchronize(s));
        double t[5];
        for (double& v : t) v = timed();
        std::sort(t, t + 5);
        return t[2];
    }
    void setFrames(int f) { frames_ = f; }
    int frames() const { return frames_; }

private:
    void issue(int k)
    {
        const FrameInput in{src_[k % src_.size()].data(), luts_.data(), &dst_[k % inflight_]};
        plan_.run({in}, streams_[k % inflight_], useGraph_);
    }
    double timed()
    {
        PS_CUDA(cudaEventRecord(t0_, streams_[0]));
        for (int s = 1; s < inflight_; s++) PS_CUDA(cudaStreamWaitEvent(streams_[s], t0_, 0));
        for (int k = 0; k < frames_; k++) issue(k);
        for (int s = 1; s < inflight_; s++) {
            PS_CUDA(cudaEventRecord(ends_[s], streams_[s]));
            PS_CUDA(cudaStreamWaitEvent(streams_[0], ends_[s], 0));
        }
        PS_CUDA(cudaEventRecord(t1_, streams_[0]));
        PS_CUDA(cudaEventSynchronize(t1_));
        float ms = 0;
        PS_CUDA(cudaEventElapsedTime(&ms, t0_, t1_));
        return (double)ms / frames_;
    }

    Rig& rig_;
    Plan& plan_;
    int frames_, inflight_;
    bool useGraph_;
    std::vector<std::vector<ps_image>> src_;  // per state slot: the cameras' inputs
    std::vector<ps_image> dst_;
    std::vector<uint8_t> luts_;
    std::vector<DevBuf> out_;
    std::vector<cudaStream_t> streams_;
    std::vector<cudaEvent_t> ends_;
    cudaEvent_t t0_ = nullptr, t1_ = nullptr;
};

// The values worth timing for each knob of `cur` (its own value excluded).
std::vector<LaunchShape> neighbours(const Rig& rig, const LaunchShape& cur, int knob)
{
    std::vector<LaunchShape> out;
    const int L = rig.numLevels();
    int curDown = 0, curBlend = 0;
    rig.tailSplit(cur.tailMaxItems, &curDown, &curBlend);
    const bool tail = curDown <= L || curBlend <= L;
    switch (knob) {
    case 0: {  // the tail split: one value per distinct split
        std::vector<std::pair<int, int>> seen{{curDown, curBlend}};
        for (int v : {0, 2, 4, 8, 16, 32, 64, 128, 256}) {
            int d = 0, b = 0;
            rig.tailSplit(v, &d, &b);
            if (std::find(seen.begin(), seen.end(), std::make_pair(d, b)) != seen.end()) continue;
            seen.push_back({d, b});
            LaunchShape s = cur;
            s.tailMaxItems = v;
            out.push_back(s);
            // the blend levels a smaller tail hands back run best as half tiles
            // together with it, so the split is also tried with those levels in
            // k_blend_small (each knob alone can measure slower than the pair)
            int most = 0;
            for (int j = std::max(1, b); j < curBlend; j++) most = std::max(most, rig.numBlendItems(j));
            if (most > cur.smallBlendMaxItems && most <= 512) {
                s.smallBlendMaxItems = most;
                out.push_back(s);
            }
        }
        break;
    }
    case 1:  // whole or half tiles for the tail's blend levels above 0
        if (tail && curBlend <= L && L >= 1) {
            LaunchShape s = cur;
            s.tailHalf = 1 - cur.tailHalf;
            out.push_back(s);
        }
        break;
    case 2:  // tail cluster width
        if (tail && tailClusterMax() > 8) {
            LaunchShape s = cur;
            s.tailCluster = cur.tailCluster == 8 ? 0 : 8;
            out.push_back(s);
        }
        break;
    case 6: {  // the blend levels run as half tiles by k_blend_small: one value per distinct set
        auto smallLevels = [&](int v) {
            int c = 0;
            for (int j = 1; j < curBlend; j++) c += rig.numBlendItems(j) <= v;
            return c;
        };
        std::vector<int> seen{smallLevels(cur.smallBlendMaxItems)};
        for (int v : {0, 32, 64, 128, 256, 512, 1024, 2048, 4096}) {
            const int c = smallLevels(v);
            if (std::find(seen.begin(), seen.end(), c) != seen.end()) continue;
            seen.push_back(c);
            LaunchShape s = cur;
            s.smallBlendMaxItems = v;
            out.push_back(s);
        }
        break;
    }
    case 7: {  // near-tie remap pixels: a second launch, or inside k_remap
        LaunchShape s = cur;
        s.remapDefer = 1 - cur.remapDefer;
        out.push_back(s);
        break;
    }
    default: {  // CTAs per SM of k_blend (3), k_pyrdown (4), k_remap (5)
        const int k = 5 - knob;
        const int resident = residentCtasPerSm(k);
        for (int v = 0; v < resident; v++) {
            if (v == cur.ctasPerSm[k] || (v == 0 && cur.ctasPerSm[k] >= resident)) continue;
            LaunchShape s = cur;
            s.ctasPerSm[k] = v;
            out.push_back(s);
        }
        break;
    }
    }
    return out;
}

}  // namespace

LaunchShape autotune(Rig& rig, Plan& plan, int framesPerTrial, int inflight, bool useGraph, bool force,
                     TuneReport* rep)
{
    NvtxRange range("ps.autotune");
    if (!rig.ready()) fail(PS_ESTATE, "render not prepared");
    if (rig.linear()) fail(PS_EINVAL, "the linear-blend mode has one launch and nothing to tune");
    if (framesPerTrial < 0 || framesPerTrial > 10000) fail(PS_EINVAL, "frames_per_trial must be in 0..10000");
    if (inflight < 0 || inflight > rig.slots())
        fail(PS_EINVAL, "in_flight must be in 0..%d (the render's state slots)", rig.slots());
    if (framesPerTrial == 0) framesPerTrial = 20;
    if (inflight == 0) inflight = rig.slots();
    const std::string key = tuneKey(rig, inflight, useGraph);
    TuneReport report;
    if (!force) {
        std::lock_guard<std::mutex> lk(g_tuneMu);
        auto it = g_tuned.find(key);
        if (it != g_tuned.end()) {
            rig.setShape(it->second.shape);
            plan.bind({&rig});
            report = it->second.report;
            report.trials = 0;
            report.cached = true;
            if (rep) *rep = report;
            return it->second.shape;
        }
    }
    const LaunchShape start = rig.shape();
    LaunchShape best;  // the default shape is the first point
    try {
        rig.waitIdle();  // the render's earlier frames are done with the staging the trials overwrite
        Trials trials(rig, plan, framesPerTrial, inflight, useGraph);
        double tBest = trials.time(best);
        report.trials = 1;
        // at least ~4 ms of device time and eight frames per stream per timed
        // run: a short run is mostly the pipeline filling and draining, which
        // hides what a shape changes in the steady state of frames in flight
        const int want = (int)std::min(4000.0, std::max({(double)framesPerTrial, 4.0 / std::max(tBest, 1e-4),
                                                          8.0 * inflight}));
        if (want > trials.frames()) {
            trials.setFrames(want);
            tBest = trials.time(best);
            report.trials++;
        }
        report.msDefault = tBest;
        // The knobs interact: with frames in flight, dropping the tail kernel,
        // running the few-tile levels as half tiles and narrowing the blend
        // grid pay off together while each alone measures slower.  So a small
        // grid over those three seeds the descent.
        {
            std::vector<LaunchShape> seen{best};
            const int L = rig.numLevels();
            for (int tail : {0, 2, 16})
                for (int small : {0, 32, 128})
                    for (int ctas : {0, 1, 2}) {
                        LaunchShape s;
                        s.tailMaxItems = tail;
                        s.smallBlendMaxItems = small;
                        s.ctasPerSm[2] = ctas;
                        // shapes that launch the same work the same way are timed once
                        int d = 0, b = 0;
                        rig.tailSplit(tail, &d, &b);
                        int smallLevels = 0;
                        for (int j = 1; j < b && j <= L; j++) smallLevels += rig.numBlendItems(j) <= small;
                        bool dup = false;
                        for (const LaunchShape& o : seen) {
                            int od = 0, ob = 0;
                            rig.tailSplit(o.tailMaxItems, &od, &ob);
                            int os = 0;
                            for (int j = 1; j < ob && j <= L; j++) os += rig.numBlendItems(j) <= o.smallBlendMaxItems;
                            if (od == d && ob == b && os == smallLevels && o.ctasPerSm[2] == ctas) dup = true;
                        }
                        if (dup) continue;
                        seen.push_back(s);
                        const double t = trials.time(s);
                        report.trials++;
                        if (t < tBest * 0.99) {
                            tBest = t;
                            best = s;
                        }
                    }
        }
        // coordinate descent, two passes; a move must gain 1%
        for (int pass = 0; pass < 2; pass++) {
            bool moved = false;
            for (int knob : {0, 6, 1, 2, 3, 4, 5, 7})
                for (const LaunchShape& s : neighbours(rig, best, knob)) {
                    const double t = trials.time(s);
                    report.trials++;
                    if (t < tBest * 0.99) {
                        tBest = t;
                        best = s;
                        moved = true;
                    }
                }
            if (!moved) break;
        }
        report.msChosen = trials.time(best);
        report.trials++;
        if (report.msChosen > report.msDefault) {  // noise: keep the default unless it measured slower
            best = LaunchShape();
            report.msChosen = report.msDefault;
        }
    } catch (...) {
        try {
            rig.setShape(start);
            plan.bind({&rig});
        } catch (...) {
        }
        throw;
    }
    rig.setShape(best);
    plan.bind({&rig});
    {
        std::lock_guard<std::mutex> lk(g_tuneMu);
        g_tuned[key] = {best, report};
    }
    if (rep) *rep = report;
    return best;
}

}  // namespace ps
