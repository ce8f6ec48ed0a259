// ps_rig.h -- prepared per-rig device state and the launch plans that run it.
#pragma once

#include <memory>

#include "ps_internal.h"

namespace ps {

struct LevelGeom {
    int w, h, pitch;
};

// One prepared rig: pyramids, weights, maps and work lists resident on the
// device (CudaTilingMultibandBlendFast's state plus the render's maps).
class Rig {
public:
    Rig() = default;
    ~Rig();
    Rig(const Rig&) = delete;
    Rig& operator=(const Rig&) = delete;

    // CudaPanoramaRender2::prepare: maps + coverage from the camera
    // parameters; seams given, or derived by seamRule (PS_SEAMS_*).
    // highQuality 0 prepares the linear-blend mode, with blendParam the
    // Gaussian radius of the weights (RicohUtil.cpp:1174-1193).
    void prepareFromParams(const ps_photo_param* params, int n, int blendParam, int srcW, int srcH, int dstW,
                           int dstH, const uint8_t* const* seams, cudaStream_t st, int seamRule = PS_SEAMS_NEAREST_AXIS,
                           int highQuality = 1);
    // CudaTilingMultibandBlendFast::prepare: coverage masks given; seams
    // given, or getNonIntersectingMasks of the coverage when seams is NULL.
    void prepareFromMasks(const uint8_t* const* masks, const uint8_t* const* seams, int n, int W, int H,
                          int maxLevels, int minLength, cudaStream_t st);
    // Frees the resident state after the rig's runs in flight have finished.
    void clear();
    // CudaTilingMultibandBlendFast::blend(images, masks, blendImage)
    // (CudaMultibandBlend.cpp:825-893): the frames that follow are weighted by
    // n host masks (W x H, non-zero = 256) instead of the unique masks, always
    // normalised by the weight sums, and zeroed outside the masks' union.
    // masks = NULL restores the prepared unique masks.  Waits for the rig's
    // runs, rebuilds the weight pyramids and blend items, starts a new
    // generation.  Synchronises.
    void setCustomMasks(const uint8_t* const* masks, cudaStream_t st);
    bool customMasks() const { return custom_; }

    bool ready() const { return n_ > 0; }
    int numImages() const { return n_; }
    int numLevels() const { return L_; }
    bool fullMask() const { return full_ != 0; }
    int width() const { return W_; }
    int height() const { return H_; }
    int srcW() const { return srcW_; }
    int srcH() const { return srcH_; }
    bool hasMaps() const { return hasMaps_; }
    bool linear() const { return linear_; }
    const LinearItem* linearItems() const { return dLinear_.as<LinearItem>(); }
    int numLinearItems() const { return numLinear_; }
    uint64_t generation() const { return gen_; }
    long long residentBytes() const;
    // resident bytes a rig of this shape would hold (no allocation)
    static long long estimateBytes(const ps_photo_param* params, int n, int blendParam, int srcW, int srcH,
                                   int dstW, int dstH, int slots = kIoSlots, bool mapFree = false);
    // Map-free remap (next prepare): no resident maps; the remap computes
    // each source coordinate in fp32 (within +-1 of the exact level 0).
    // Taken by itself when even one slot with maps does not fit.
    void setMapFree(bool on) { mapFreeWanted_ = on; }
    bool mapFree() const { return mapFree_; }

    // Device staging of host frames and of a host canvas: one set per state
    // slot, so consecutive renders with host buffers overlap their copies (slot 0's
    // frame buffers are also the ones ps_render_get_input_buffer exposes).
    static constexpr int kIoSlots = PS_MAX_IN_FLIGHT;  // most state slots a rig keeps
    // state slots of the next prepare (1..kIoSlots; default kIoSlots)
    void setSlots(int n) { slotsWanted_ = n < 1 ? 1 : (n > kIoSlots ? kIoSlots : n); }
    int slots() const { return slots_; }
    // the last prepare found too little free device memory for the slots
    // asked for and took fewer (the reference's low-memory path)
    bool lowMemory() const { return lowMemory_; }
    // device bytes the next prepare may take for the render (0: no limit
    // but the free memory)
    void setMemoryBudget(long long bytes) { budget_ = bytes > 0 ? bytes : 0; }
    uint8_t* inputBuffer(int cam, int slot = 0) const
    {
        return inputs_.as<uint8_t>() + ((size_t)slot * n_ + cam) * inPitch_ * srcH_;
    }
    long long inputPitch() const { return inPitch_; }
    // Staging of decoder frames (YUV420P / NV12 host planes, 1.5 bytes per
    // pixel, packed: Y, then U and V or UV), one set per state slot;
    // allocated by the first render with planar sources.
    void ensurePlanar()
    {
        if (!planar_.get()) planar_.alloc((size_t)slots_ * n_ * planarBytes());
    }
    size_t planarBytes() const { return (size_t)srcW_ * srcH_ * 3 / 2; }
    uint8_t* planarBuffer(int cam, int slot) const
    {
        return planar_.as<uint8_t>() + ((size_t)slot * n_ + cam) * planarBytes();
    }
    uint8_t* outputBuffer(int slot = 0) const { return output_.as<uint8_t>() + (size_t)slot * W_ * H_ * 4; }
    int* statusWord() const { return status_.as<int>(); }
    // The status bits the kernels set since the last call (bit 4: a bounded
    // wait of a blend kernel ran out), read and cleared after the rig's runs
    // have finished.
    int takeStatus();
    // Failure-path test of the bounded waits: with polls > 0 every blend
    // launch of this rig makes one wait of that many polls on a barrier that
    // nothing completes, which therefore runs out.  0 (the default) is off.
    // Waits for the rig's runs; the next run re-records its launches.
    void setWaitProbe(int polls);
    int waitProbe() const { return probe_; }

    void exportState(int what, int cam, int level, void* host, long long bytes) const;
    void exportCollapsed(int level, int16_t* host, long long bytes, cudaStream_t st) const;

    // Per-frame state slots: the Gaussian and collapsed pyramids, the I/O
    // staging and the device descriptor that points at them come in
    // slots() copies, so that many frames of one rig can be in flight.  Runs take
    // slots in turn.  slotComputed(s) follows the last kernels that used
    // slot s (its pyramids and input staging are free again);
    // slotDownloaded(s) follows the copy out of its output staging.
    int acquireSlot()
    {
        const int s = nextSlot_;
        nextSlot_ = (s + 1) % slots_;
        lastSlot_ = s;
        return s;
    }
    int peekSlot() const { return nextSlot_; }
    cudaEvent_t slotComputed(int slot) { return slotEvent(slotComputed_[slot]); }
    cudaEvent_t slotDownloaded(int slot) { return slotEvent(slotDownloaded_[slot]); }
    // Waits for every run that used this rig, whatever plan issued it (each
    // records its slot's events after the kernels and after the download).
    // Unlike a device-wide synchronise it leaves other work alone, such as a
    // capture in progress on another thread.
    void waitIdle();
    // The same, for teardown: errors of the runs are dropped, not thrown.
    void waitIdleQuiet() noexcept;

    // building blocks of launch plans
    const RigDev* deviceDesc(int slot = 0) const { return dDesc_.as<RigDev>() + slot; }
    const RemapItem* remapItems() const { return dRemap_.as<RemapItem>(); }
    int numRemapItems() const { return (int)hRemap_.size(); }
    const DownItem* downItems(int level) const { return dDown_.as<DownItem>() + downOff_[level]; }
    int numDownItems(int level) const { return downCnt_[level]; }
    const BlendItem* blendItems(int level) const { return dBlend_.as<BlendItem>() + blendOff_[level]; }
    int numBlendItems(int level) const { return blendCnt_[level]; }
    // Launch shape (tail split, tail cluster and tile split, CTAs per SM).
    // Set before prepare, it applies at prepare; set after, it waits for the
    // rig's runs to finish (waitIdle), rewrites the descriptors and starts a
    // new generation.
    void setShape(const LaunchShape& s);
    const LaunchShape& shape() const { return shape_; }
    // the tail levels a tail_max_items value gives: pyrDown down..L, blend L..blend
    void tailSplit(int maxItems, int* down, int* blend) const;
    // pyrDown levels tailDown()..L and blend levels L..tailBlend() run in the tail kernel
    int tailDown() const { return tailDown_; }
    int tailBlend() const { return tailBlend_; }
    bool hasTail() const { return tailDown_ <= L_ || tailBlend_ <= L_; }

    // blender input: int16x4 / uint8x4 device images -> level 0 of a slot (checks)
    void imagesToLevel0(const void* const* images, const long long* pitches, int fmt, int slot, cudaStream_t st);
    // the same for one camera (CudaTilingMultibandBlendFast::tile), and a
    // camera left out of a tiled blend (its level 0 all zero: its Laplacians
    // vanish, so it contributes nothing, while its weights still count)
    void imageToLevel0(const void* image, long long pitch, int fmt, int cam, int slot, cudaStream_t st);
    void zeroLevel0(int cam, int slot, cudaStream_t st);
    // device bytes a blender of this size holds at most (any coverage)
    static long long estimateBlenderBytes(int W, int H, int n, int maxLevels, int slots = kIoSlots);

    // Bytes a step must move at minimum (each input / output element once,
    // no halo re-reads): kind 0 remap, 1 pyrDown to `level`, 2 blend of
    // `level`, 3 the tail, 4 the linear-blend render.
    double stepBytes(int kind, int level) const;
    // Algorithmic bytes of one stitched frame (inputs, maps, weights, alpha
    // divisors, output; all pyramid levels are intermediate and count 0):
    //   sum_i Ws*Hs*bin + sum_i C_i*8 + sum_ij K_ij*2 + sum_i,j>=1 A_ij*4 + Wc*Hc*bout
    double algorithmicBytes(int bin, int bout) const;

private:
    struct LevelBufs {
        DevBuf G[kIoSlots], Wt, Am, C[kIoSlots];
    };
    static cudaEvent_t slotEvent(cudaEvent_t& e);
    void setGeometry(int n, int W, int H, int L);
    void preparePyramids(const uint8_t* covDev, const uint8_t* seamDev, const float* xmapDev, const float* ymapDev,
                         cudaStream_t st);
    void prepareLinear(const uint8_t* covDev, const uint8_t* seamDev, const float* xmapDev, const float* ymapDev,
                       int radius, cudaStream_t st);
    void writeDescriptors(cudaStream_t st);
    bool encodeTensorMaps();  // tmaps_ for every slot and level; false when the driver cannot
    void toLevel0(const void* const* images, const long long* pitches, int fmt, int cam0, int count, int slot,
                  cudaStream_t st);
    void buildBlendState(const uint8_t* uniSrcDev, bool custom, cudaStream_t st);

    int n_ = 0, W_ = 0, H_ = 0, L_ = 0, full_ = 0, srcW_ = 0, srcH_ = 0;
    bool hasMaps_ = false, linear_ = false, custom_ = false, lowMemory_ = false;
    bool mapFree_ = false, mapFreeWanted_ = false;
    std::vector<RemapDev> hParams_;  // the cameras' Remap parameters of the last prepare
    DevBuf camsF_, covTiles_;
    int nextSlot_ = 0, lastSlot_ = 0, slots_ = kIoSlots, slotsWanted_ = kIoSlots, probe_ = 0;
    cudaEvent_t slotComputed_[kIoSlots] = {}, slotDownloaded_[kIoSlots] = {};
    int numLinear_ = 0;
    DevBuf dLinear_, linW_;
    uint64_t gen_ = 0;
    std::vector<LevelGeom> geom_;
    LevelBufs lv_[PS_MAX_LEVELS + 1];
    DevBuf maps_, union_, inputs_, output_, covDev_, status_, imgArgs_, planar_;
    long long inPitch_ = 0, budget_ = 0;
    DevBuf dDesc_, dRemap_, dDown_, dBlend_, dCams_;
    DevBuf tmaps_;  // slots x (L + 1) x kTmapsPerLevel CUtensorMap
    std::vector<RemapItem> hRemap_;
    int downOff_[PS_MAX_LEVELS + 1] = {}, downCnt_[PS_MAX_LEVELS + 1] = {};
    int blendOff_[PS_MAX_LEVELS + 1] = {}, blendCnt_[PS_MAX_LEVELS + 1] = {};
    int tailDown_ = 1, tailBlend_ = 1;
    LaunchShape shape_;
    RigDev hDesc_ = {};  // slot-independent part of the descriptors
    std::vector<uint8_t> covBits_, seamBits_;  // host copies for exports (1 bit / pixel)
    std::vector<DownItem> hDown_;
    std::vector<BlendItem> hBlend_;
    std::vector<uint8_t> hCams_;
    long long covCount_ = 0, weightCount_ = 0, alphaCount_ = 0;  // non-zero pixels, all cameras / levels
};

// Per-launch CUDA-event timing of the steps of a plan (non-graph runs only).
class Profiler {
public:
    ~Profiler();
    void enable(bool on);
    bool on() const { return on_; }
    void record(int kind, int level, double bytes, cudaEvent_t a, cudaEvent_t b);
    cudaEvent_t event();
    // aggregate of finished launches of (kind, level); level -1 = all levels
    void read(int kind, int level, long long* launches, double* ms, double* bytes);

private:
    struct Rec { int kind, level; double bytes; cudaEvent_t a, b; };
    struct Agg { long long launches = 0; double ms = 0, bytes = 0; };
    void collect();
    bool on_ = false;
    std::vector<Rec> recs_;
    std::vector<cudaEvent_t> free_;
    std::vector<std::pair<std::pair<int, int>, Agg>> agg_;
};

// Per-frame inputs of one rig in a plan.
struct FrameInput {
    const ps_image* src;      // numImages images, or nullptr when level 0 is already written
    const uint8_t* luts;      // n*768 host bytes or nullptr (identity)
    const ps_image* dst;      // BGR canvas, or nullptr when ydst is given
    const ps_planar_image* ydst = nullptr;  // YUV420P / NV12 planes instead of dst
    const ps_planar_image* psrc = nullptr;  // numImages decoder frames (YUV420P / NV12) instead of src
};

// The launch sequence for a set of rigs: one remap launch, one pyrDown
// launch per level, one blend launch per level; each launch runs the work
// items of every rig (one segment per rig).  Optionally captured into a CUDA
// graph on first run.
class Plan {
public:
    Plan() = default;
    explicit Plan(const std::vector<Rig*>& rigs) { bind(rigs); }
    ~Plan();
    Plan(const Plan&) = delete;
    Plan& operator=(const Plan&) = delete;
    // (re)build the steps for this set of rigs, reusing buffers when they fit
    void bind(const std::vector<Rig*>& rigs);
    // stage frame arguments, upload host inputs, run, download host outputs
    void run(const std::vector<FrameInput>& in, cudaStream_t st, bool useGraph, Profiler* prof = nullptr);
    int launchesPerRun() const { return (int)steps_.size(); }
    bool matches(const std::vector<Rig*>& rigs) const;

private:
    struct Step {
        int kind;  // 0 remap, 1 pyrDown, 2 blend, 3 tail, 4 linear-blend render, 6 few-tile blend,
                   // 7 the exact recompute of the remap tiles near rounding ties
        int segOff, nsegs, total;
        int level;      // level of the first rig in the step
        double bytes;   // algorithmic bytes of the step (all rigs)
        bool early = false;  // a blend step after the first: only C levels were written by the launch before
    };
    // Per-run state in kIoSlots copies: run k uses slot k % kIoSlots, so while
    // run k computes, run k + 1 uploads and run k - 1 downloads.
    struct IoSlot {
        DevBuf dArgs;   // [FrameDev x nr][LUTs][Segment x nseg]
        HostBuf stage;  // pinned staging copy of dArgs
        DevBuf ties;    // the remap's list of near-tie pixels for k_remap_fix
        cudaGraphExec_t graph = nullptr;
        int graphFmt = 0;  // the sources' format the graph's remap was specialised for (0: any)
        cudaEvent_t argsCopied = nullptr, computed = nullptr, downloaded = nullptr;
        bool used = false;
    };
    // srcFmt: the format every source of the run shares (0: mixed)
    void launchAll(const IoSlot& slot, cudaStream_t st, int srcFmt, Profiler* prof = nullptr);
    void dropGraph();
    void ensureStreams();
    void quiesce();

    std::vector<Rig*> rigs_;
    std::vector<uint64_t> gens_;
    std::vector<Step> steps_;
    std::vector<Segment> segs_;      // frame pointers hold offsets into the args block
    std::vector<int> segRig_;        // rig of each segment (its descriptor depends on the rig's slot)
    std::vector<size_t> lutOff_;
    size_t segOff_ = 0, counterOff_ = 0, stageBytes_ = 0;
    int maxCams_ = 0;
    int tailCluster_ = 0, perSm_[3] = {0, 0, 0};  // launch widths (from the rigs' shapes)
    bool remapDefer_ = true;                      // k_remap lists near-tie pixels for k_remap_fix
    int probe_ = 0;                                // wait probe of k_blend (Rig::setWaitProbe)
    IoSlot io_[Rig::kIoSlots];
    int nextIo_ = 0;
    // copy-in, compute and copy-out streams (non-blocking), the capture stream
    cudaStream_t sIn_ = nullptr, sComp_[Rig::kIoSlots] = {}, sOut_ = nullptr, capStream_ = nullptr;
    cudaEvent_t callerEv_ = nullptr;
};

// The autotuner (ps_tune.cpp): times launch shapes on a prepared rig by
// a grid over the tail split, the half-tile levels and the blend's CTAs per
// SM, then coordinate descent from the best of it (tail split, the levels run as
// half tiles by k_blend_small, tail tile split, tail cluster width, CTAs per
// SM of k_blend, k_pyrdown, k_remap), frames
// issued round-robin on `inflight` streams, and leaves the fastest set on
// the rig and bound to the plan.  Results are kept per rig geometry, GPU and
// concurrency, so a later call for the same geometry times nothing unless
// forced.  Blocks until done.
struct TuneReport {
    double msDefault = 0, msChosen = 0;  // ms per frame of the default and the chosen shape
    int trials = 0;                      // timed runs
    bool cached = false;
};
LaunchShape autotune(Rig& rig, Plan& plan, int framesPerTrial, int inflight, bool useGraph, bool force,
                     TuneReport* rep);

}  // namespace ps
