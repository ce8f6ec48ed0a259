// ps_capi.cpp -- the extern "C" boundary: validation, status codes, the
// thread-local error text, and the objects behind the opaque handles.
#include <algorithm>
#include <cmath>
#include <map>
#include <memory>
#include <mutex>
#include <set>

#include "ps_rig.h"

using ps::fail;

struct ps_render {
    ps::Rig rig;
    std::unique_ptr<ps::Plan> plan;
    ps::Profiler prof;
    bool useGraph = true;
    int seamRule = PS_SEAMS_NEAREST_AXIS;
};

struct ps_blender {
    ps::Rig rig;
    std::unique_ptr<ps::Plan> plan;
    // begin / tile / end in progress: the state slot the tiles go to and the
    // cameras tiled so far
    bool tiling = false;
    int tileSlot = 0;
    uint64_t tiled = 0;
};

namespace {

thread_local std::string t_err;

template <class F>
int guarded(F&& f)
{
    try {
        f();
        return PS_OK;
    } catch (const ps::Error& e) {
        t_err = e.what();
        return e.code;
    } catch (const std::bad_alloc&) {
        t_err = "host allocation failed";
        return PS_ENOMEM;
    } catch (const std::exception& e) {
        t_err = e.what();
        return PS_EINVAL;
    } catch (...) {
        t_err = "unknown error";
        return PS_EINVAL;
    }
}

inline cudaStream_t toStream(void* s) { return static_cast<cudaStream_t>(s); }

int bpp(int fmt) { return fmt == PS_FMT_BGR24 ? 3 : 4; }

void checkImage(const ps_image* im, int w, int h, const char* what, int idx)
{
    if (!im) fail(PS_EINVAL, "%s[%d] is NULL", what, idx);
    if (!im->data) fail(PS_EINVAL, "%s[%d]: data is NULL", what, idx);
    if (im->format != PS_FMT_BGR24 && im->format != PS_FMT_BGR32)
        fail(PS_EINVAL, "%s[%d]: format %d is neither BGR24 nor BGR32", what, idx, im->format);
    if (im->location != PS_MEM_HOST && im->location != PS_MEM_DEVICE)
        fail(PS_EINVAL, "%s[%d]: location %d unknown", what, idx, im->location);
    // source/Task/RicohUtil.cpp:1222-1236
    if (im->width != w || im->height != h)
        fail(PS_EINVAL, "%s[%d] size (%d, %d), not equal to (%d, %d)", what, idx, im->width, im->height, w, h);
    if (im->pitch < (long long)w * bpp(im->format)) fail(PS_EINVAL, "%s[%d]: pitch %lld too small", what, idx, im->pitch);
    if (im->location == PS_MEM_DEVICE && im->format == PS_FMT_BGR32 &&
        ((reinterpret_cast<uintptr_t>(im->data) & 3) || (im->pitch & 3)))
        fail(PS_EINVAL, "%s[%d]: device BGR32 images need 4-byte aligned data and pitch", what, idx);
}

void checkFrame(const ps::Rig& rig, const ps_image* src, int numSrc, const uint8_t* luts, int numLuts,
                const ps_image* dst)
{
    if (!rig.ready()) fail(PS_ESTATE, "have not prepared or prepare failed before");
    if (!rig.hasMaps()) fail(PS_ESTATE, "prepared without camera parameters");
    if (!src || numSrc != rig.numImages())
        fail(PS_EINVAL, "%d source images given, %d cameras prepared", numSrc, rig.numImages());
    for (int i = 0; i < numSrc; i++) {
        checkImage(&src[i], rig.srcW(), rig.srcH(), "src", i);
        if (src[i].format != src[0].format) fail(PS_EINVAL, "src[%d]: all sources must share one format", i);
    }
    if (luts && numLuts != rig.numImages())
        fail(PS_EINVAL, "%d look-up tables given, %d cameras prepared (each 3 x 256 bytes)", numLuts, rig.numImages());
    checkImage(dst, rig.width(), rig.height(), "dst", 0);
}

// A planar YUV420P / NV12 view of w x h (both even).
void checkPlanar(const ps_planar_image* im, int w, int h, const char* what)
{
    if (!im) fail(PS_EINVAL, "%s is NULL", what);
    if (im->format != PS_FMT_YUV420P && im->format != PS_FMT_NV12)
        fail(PS_EINVAL, "%s: format %d is neither YUV420P nor NV12", what, im->format);
    if (im->location != PS_MEM_HOST && im->location != PS_MEM_DEVICE)
        fail(PS_EINVAL, "%s: location %d unknown", what, im->location);
    if (im->width != w || im->height != h)
        fail(PS_EINVAL, "%s size (%d, %d), not equal to (%d, %d)", what, im->width, im->height, w, h);
    // CV_Assert((rows & 1) == 0 && (cols & 1) == 0), ImageProc.cu:123,143
    if (w <= 0 || h <= 0 || (w & 1) || (h & 1)) fail(PS_EINVAL, "%s: size (%d, %d) must be positive and even", what, w, h);
    const int planes = im->format == PS_FMT_NV12 ? 2 : 3;
    const long long minPitch[3] = {w, im->format == PS_FMT_NV12 ? w : w / 2, w / 2};
    for (int k = 0; k < planes; k++) {
        if (!im->planes[k]) fail(PS_EINVAL, "%s: plane %d is NULL", what, k);
        if (im->pitches[k] < minPitch[k]) fail(PS_EINVAL, "%s: plane %d pitch %lld too small", what, k, im->pitches[k]);
    }
}

// Launch plans of batches, keyed by the rigs they run.
std::mutex g_planMu;
std::map<std::vector<ps::Rig*>, std::unique_ptr<ps::Plan>> g_batchPlans;

void purgePlans(const ps::Rig* rig)
{
    std::lock_guard<std::mutex> lk(g_planMu);
    for (auto it = g_batchPlans.begin(); it != g_batchPlans.end();) {
        if (std::find(it->first.begin(), it->first.end(), rig) != it->first.end()) it = g_batchPlans.erase(it);
        else ++it;
    }
}

}  // namespace

void ps::setLastError(const std::string& msg) { t_err = msg; }

extern "C" {

const char* ps_last_error(void) { return t_err.c_str(); }
const char* ps_version(void) { return "panostitch-gb300 0.1 (sm_103a)"; }

// ---- render ----------------------------------------------------------------------
int ps_render_create(ps_render** out)
{
    return guarded([&] {
        if (!out) fail(PS_EINVAL, "out is NULL");
        *out = new ps_render();
    });
}

void ps_render_destroy(ps_render* r)
{
    if (!r) return;
    purgePlans(&r->rig);
    delete r;
}

static int prepareRender(ps_render* r, const ps_photo_param* params, int num, int hq, int blendParam, int srcW,
                         int srcH, int dstW, int dstH, const uint8_t* const* seams, void* stream)
{
    return guarded([&] {
        if (!r) fail(PS_EINVAL, "render is NULL");
        purgePlans(&r->rig);
        r->plan.reset();
        r->rig.clear();
        // source/Task/RicohUtil.cpp:1120-1193: non-zero = multiband, 0 = linear blend
        r->rig.prepareFromParams(params, num, blendParam, srcW, srcH, dstW, dstH, seams, toStream(stream),
                                 r->seamRule, hq != 0);
        r->plan.reset(new ps::Plan({&r->rig}));
    });
}

int ps_load_photo_params(const char* path, ps_photo_param* params, int capacity, int* num)
{
    return guarded([&] {
        if (!path || !num || capacity < 0 || (capacity > 0 && !params)) fail(PS_EINVAL, "NULL argument");
        const std::vector<ps_photo_param> p = ps::loadPhotoParams(path);
        *num = (int)p.size();
        for (int i = 0; i < capacity && i < (int)p.size(); i++) params[i] = p[i];
    });
}

int ps_render_prepare_file(ps_render* r, const char* path, int high_quality_blend, int blend_param, int src_w,
                           int src_h, int dst_w, int dst_h, void* stream)
{
    std::vector<ps_photo_param> p;
    const int st = guarded([&] {
        if (!r || !path) fail(PS_EINVAL, "NULL argument");
        p = ps::loadPhotoParams(path);
        if (p.empty()) fail(PS_EINVAL, "load photo params failed");  // RicohUtil.cpp:1111-1116
    });
    if (st != PS_OK) {
        if (r) ps_render_clear(r);
        return st;
    }
    return ps_render_prepare(r, p.data(), (int)p.size(), high_quality_blend, blend_param, src_w, src_h, dst_w, dst_h,
                             stream);
}

int ps_render_prepare(ps_render* r, const ps_photo_param* params, int num_params, int high_quality_blend,
                      int blend_param, int src_w, int src_h, int dst_w, int dst_h, void* stream)
{
    return prepareRender(r, params, num_params, high_quality_blend, blend_param, src_w, src_h, dst_w, dst_h,
                         nullptr, stream);
}

int ps_render_prepare_with_seams(ps_render* r, const ps_photo_param* params, int num_params,
                                 int high_quality_blend, int blend_param, int src_w, int src_h, int dst_w,
                                 int dst_h, const uint8_t* const* seam_masks, void* stream)
{
    if (!seam_masks) {
        t_err = "seam_masks is NULL";
        return PS_EINVAL;
    }
    return prepareRender(r, params, num_params, high_quality_blend, blend_param, src_w, src_h, dst_w, dst_h,
                         seam_masks, stream);
}

int ps_render_render(ps_render* r, const ps_image* src, int num_src, const uint8_t* luts, int num_luts,
                     ps_image* dst, void* stream)
{
    return guarded([&] {
        if (!r) fail(PS_EINVAL, "render is NULL");
        checkFrame(r->rig, src, num_src, luts, num_luts, dst);
        if (!r->plan || !r->plan->matches({&r->rig})) r->plan.reset(new ps::Plan({&r->rig}));
        r->plan->run({ps::FrameInput{src, luts, dst}}, toStream(stream), r->useGraph, &r->prof);
    });
}

int ps_render_profile(ps_render* r, int enable)
{
    return guarded([&] {
        if (!r) fail(PS_EINVAL, "render is NULL");
        r->prof.enable(enable != 0);
    });
}

int ps_render_profile_read(ps_render* r, int kind, int level, long long* launches, double* total_ms, double* bytes)
{
    return guarded([&] {
        if (!r) fail(PS_EINVAL, "render is NULL");
        if (kind < 0 || kind > 7) fail(PS_EINVAL, "kind %d not in 0..7", kind);
        r->prof.read(kind, level, launches, total_ms, bytes);
    });
}

int ps_render_launches_per_frame(const ps_render* r)
{
    return r && r->plan ? r->plan->launchesPerRun() : 0;
}

double ps_render_algorithmic_bytes(const ps_render* r, int bytes_in_per_px, int bytes_out_per_px)
{
    if (!r || !r->rig.ready()) return -1.0;
    return r->rig.algorithmicBytes(bytes_in_per_px, bytes_out_per_px);
}

// ---- launch shapes ------------------------------------------------------------
namespace {

ps::LaunchShape fromAbi(const ps_launch_shape& s)
{
    ps::LaunchShape o;
    o.tailMaxItems = s.tail_max_items;
    o.tailCluster = s.tail_cluster;
    o.tailHalf = s.tail_half_tiles;
    for (int k = 0; k < 3; k++) o.ctasPerSm[k] = s.ctas_per_sm[k];
    o.smallBlendMaxItems = s.small_blend_max_items;
    o.remapDefer = s.remap_defer_ties;
    return o;
}

void toAbi(const ps::LaunchShape& s, ps_launch_shape* o)
{
    o->tail_max_items = s.tailMaxItems;
    o->tail_cluster = s.tailCluster;
    o->tail_half_tiles = s.tailHalf;
    for (int k = 0; k < 3; k++) o->ctas_per_sm[k] = s.ctasPerSm[k];
    o->small_blend_max_items = s.smallBlendMaxItems;
    o->remap_defer_ties = s.remapDefer;
}

}  // namespace

int ps_render_set_launch_shape(ps_render* r, const ps_launch_shape* shape)
{
    return guarded([&] {
        if (!r || !shape) fail(PS_EINVAL, "NULL argument");
        r->rig.setShape(fromAbi(*shape));
    });
}

int ps_render_get_launch_shape(const ps_render* r, ps_launch_shape* shape)
{
    return guarded([&] {
        if (!r || !shape) fail(PS_EINVAL, "NULL argument");
        toAbi(r->rig.shape(), shape);
    });
}

int ps_render_autotune(ps_render* r, int frames_per_trial, int in_flight, int force, ps_launch_shape* chosen,
                       ps_tune_report* report)
{
    return guarded([&] {
        if (!r) fail(PS_EINVAL, "render is NULL");
        if (!r->rig.ready()) fail(PS_ESTATE, "render not prepared");
        if (!r->plan || !r->plan->matches({&r->rig})) r->plan.reset(new ps::Plan({&r->rig}));
        ps::TuneReport rep;
        const ps::LaunchShape s =
            ps::autotune(r->rig, *r->plan, frames_per_trial, in_flight, r->useGraph, force != 0, &rep);
        if (chosen) toAbi(s, chosen);
        if (report) {
            report->ms_per_frame_default = rep.msDefault;
            report->ms_per_frame_chosen = rep.msChosen;
            report->trials = rep.trials;
            report->cached = rep.cached ? 1 : 0;
        }
    });
}

int ps_render_render_yuv(ps_render* r, const ps_image* src, int num_src, const uint8_t* luts, int num_luts,
                         const ps_planar_image* dst, void* stream)
{
    return guarded([&] {
        if (!r) fail(PS_EINVAL, "render is NULL");
        if (!r->rig.ready()) fail(PS_ESTATE, "have not prepared or prepare failed before");
        if (r->rig.linear()) fail(PS_EINVAL, "the linear-blend mode writes BGR only; use ps_cvt_bgr32_to_yuv");
        checkPlanar(dst, r->rig.width(), r->rig.height(), "dst");
        ps_image probe = {dst->planes[0], (long long)r->rig.width() * 4, r->rig.width(), r->rig.height(),
                          PS_FMT_BGR32, PS_MEM_DEVICE};  // only for the shared source / LUT checks
        checkFrame(r->rig, src, num_src, luts, num_luts, &probe);
        if (!r->plan || !r->plan->matches({&r->rig})) r->plan.reset(new ps::Plan({&r->rig}));
        r->plan->run({ps::FrameInput{src, luts, nullptr, dst}}, toStream(stream), r->useGraph, &r->prof);
    });
}

int ps_render_set_frames_in_flight(ps_render* r, int n)
{
    return guarded([&] {
        if (!r) fail(PS_EINVAL, "render is NULL");
        if (n < 1 || n > PS_MAX_IN_FLIGHT) fail(PS_EINVAL, "frames in flight %d not in 1..%d", n, PS_MAX_IN_FLIGHT);
        r->rig.setSlots(n);
    });
}

int ps_render_get_frames_in_flight(const ps_render* r) { return r && r->rig.ready() ? r->rig.slots() : 0; }

int ps_render_set_memory_budget(ps_render* r, long long bytes)
{
    return guarded([&] {
        if (!r) fail(PS_EINVAL, "render is NULL");
        if (bytes < 0) fail(PS_EINVAL, "budget %lld is negative", bytes);
        r->rig.setMemoryBudget(bytes);
    });
}

int ps_render_is_low_memory(const ps_render* r) { return r && r->rig.ready() && r->rig.lowMemory() ? 1 : 0; }

int ps_render_set_map_free(ps_render* r, int enable)
{
    return guarded([&] {
        if (!r) fail(PS_EINVAL, "render is NULL");
        r->rig.setMapFree(enable != 0);
    });
}

int ps_render_is_map_free(const ps_render* r) { return r && r->rig.ready() && r->rig.mapFree() ? 1 : 0; }

int ps_render_render_planar(ps_render* r, const ps_planar_image* src, int num_src, const uint8_t* luts,
                            int num_luts, const ps_image* dst, const ps_planar_image* ydst, void* stream)
{
    return guarded([&] {
        if (!r) fail(PS_EINVAL, "render is NULL");
        const ps::Rig& rig = r->rig;
        if (!rig.ready()) fail(PS_ESTATE, "have not prepared or prepare failed before");
        if (!rig.hasMaps()) fail(PS_ESTATE, "prepared without camera parameters");
        if (!src || num_src != rig.numImages())
            fail(PS_EINVAL, "%d source frames given, %d cameras prepared", num_src, rig.numImages());
        for (int i = 0; i < num_src; i++) checkPlanar(&src[i], rig.srcW(), rig.srcH(), "src");
        if (luts && num_luts != rig.numImages())
            fail(PS_EINVAL, "%d look-up tables given, %d cameras prepared (each 3 x 256 bytes)", num_luts,
                 rig.numImages());
        if ((dst == nullptr) == (ydst == nullptr)) fail(PS_EINVAL, "give exactly one of dst and ydst");
        if (dst) {
            checkImage(dst, rig.width(), rig.height(), "dst", 0);
        } else {
            if (rig.linear()) fail(PS_EINVAL, "the linear-blend mode writes BGR only; use ps_cvt_bgr32_to_yuv");
            checkPlanar(ydst, rig.width(), rig.height(), "ydst");
        }
        if (!r->plan || !r->plan->matches({&r->rig})) r->plan.reset(new ps::Plan({&r->rig}));
        ps::FrameInput in{nullptr, luts, dst, ydst};
        in.psrc = src;
        r->plan->run({in}, toStream(stream), r->useGraph, &r->prof);
    });
}

int ps_render_set_seam_rule(ps_render* r, int rule)
{
    return guarded([&] {
        if (!r) fail(PS_EINVAL, "render is NULL");
        if (rule != PS_SEAMS_NEAREST_AXIS && rule != PS_SEAMS_DISTANCE) fail(PS_EINVAL, "unknown seam rule %d", rule);
        r->seamRule = rule;
    });
}

static void setCustomMasks(ps::Rig& rig, const uint8_t* const* masks, int num, void* stream)
{
    if (!rig.ready()) fail(PS_ESTATE, "have not prepared or prepare failed before");
    if (masks && num != rig.numImages())
        fail(PS_EINVAL, "%d custom masks given, %d cameras prepared", num, rig.numImages());
    if (!masks && num != 0) fail(PS_EINVAL, "masks is NULL but num_masks = %d", num);
    rig.setCustomMasks(masks, toStream(stream));
}

int ps_render_set_custom_masks(ps_render* r, const uint8_t* const* masks, int num_masks, void* stream)
{
    return guarded([&] {
        if (!r) fail(PS_EINVAL, "render is NULL");
        setCustomMasks(r->rig, masks, num_masks, stream);
    });
}

int ps_render_set_graph(ps_render* r, int enabled)
{
    return guarded([&] {
        if (!r) fail(PS_EINVAL, "render is NULL");
        r->useGraph = enabled != 0;
    });
}

int ps_render_get_unique_masks(const ps_render* r, uint8_t* const* masks, int num)
{
    return guarded([&] {
        if (!r) fail(PS_EINVAL, "render is NULL");
        if (!r->rig.ready()) fail(PS_ESTATE, "have not prepared or prepare failed before");
        if (!masks || num != r->rig.numImages())
            fail(PS_EINVAL, "%d mask buffers given, %d cameras prepared", num, r->rig.numImages());
        const long long bytes = (long long)r->rig.width() * r->rig.height();
        for (int i = 0; i < num; i++) {
            if (!masks[i]) fail(PS_EINVAL, "mask buffer %d is NULL", i);
            r->rig.exportState(3, i, 0, masks[i], bytes);
        }
    });
}

long long ps_render_estimate_memory(const ps_photo_param* params, int num_params, int blend_param, int src_w,
                                    int src_h, int dst_w, int dst_h, int frames_in_flight)
{
    long long v = -1;
    const int st = guarded([&] {
        if (frames_in_flight < 1 || frames_in_flight > ps::Rig::kIoSlots)
            fail(PS_EINVAL, "frames_in_flight %d out of range 1..%d", frames_in_flight, ps::Rig::kIoSlots);
        v = ps::Rig::estimateBytes(params, num_params, blend_param, src_w, src_h, dst_w, dst_h, frames_in_flight);
    });
    return st == PS_OK ? v : -1;
}

int ps_render_check(ps_render* r)
{
    return guarded([&] {
        if (!r) fail(PS_EINVAL, "render is NULL");
        if (!r->rig.ready()) return;
        const int st = r->rig.takeStatus();
        if (st & 4)
            fail(PS_ETIMEOUT, "a bounded wait of a blend kernel ran out: frames rendered since the last check "
                              "may be wrong");
    });
}

int ps_render_set_wait_probe(ps_render* r, int polls)
{
    return guarded([&] {
        if (!r) fail(PS_EINVAL, "render is NULL");
        if (!r->rig.ready()) fail(PS_ESTATE, "have not prepared or prepare failed before");
        r->rig.setWaitProbe(polls);
    });
}

void ps_render_clear(ps_render* r)
{
    if (!r) return;
    purgePlans(&r->rig);
    r->plan.reset();
    r->rig.clear();
}

int ps_render_get_num_images(const ps_render* r) { return r && r->rig.ready() ? r->rig.numImages() : 0; }
int ps_render_get_num_levels(const ps_render* r) { return r && r->rig.ready() ? r->rig.numLevels() : 0; }
int ps_render_is_full_mask(const ps_render* r) { return r && r->rig.ready() && r->rig.fullMask() ? 1 : 0; }
long long ps_render_resident_bytes(const ps_render* r) { return r ? r->rig.residentBytes() : 0; }

int ps_render_get_input_buffer(ps_render* r, int cam, void** data, long long* pitch)
{
    return guarded([&] {
        if (!r || !data || !pitch) fail(PS_EINVAL, "NULL argument");
        if (!r->rig.ready() || !r->rig.hasMaps()) fail(PS_ESTATE, "not prepared");
        if (cam < 0 || cam >= r->rig.numImages()) fail(PS_EINVAL, "camera %d out of range", cam);
        *data = r->rig.inputBuffer(cam);
        *pitch = r->rig.inputPitch();
    });
}

int ps_render_export(const ps_render* r, int what, int cam, int level, void* host_out, long long bytes)
{
    return guarded([&] {
        if (!r || !host_out) fail(PS_EINVAL, "NULL argument");
        r->rig.exportState(what, cam, level, host_out, bytes);
    });
}

int ps_render_export_collapsed(const ps_render* r, int level, int16_t* host_out, long long bytes, void* stream)
{
    return guarded([&] {
        if (!r || !host_out) fail(PS_EINVAL, "NULL argument");
        r->rig.exportCollapsed(level, host_out, bytes, toStream(stream));
    });
}

// ---- batch ----------------------------------------------------------------------
int ps_render_batch(ps_render* const* renders, int num_renders, const ps_image* const* srcs,
                    const uint8_t* const* luts, ps_image* dsts, void* stream)
{
    return guarded([&] {
        if (!renders || !srcs || !dsts || num_renders <= 0) fail(PS_EINVAL, "empty batch");
        std::vector<ps::Rig*> rigs;
        std::set<ps_render*> seen;
        std::vector<ps::FrameInput> in;
        for (int k = 0; k < num_renders; k++) {
            ps_render* r = renders[k];
            if (!r) fail(PS_EINVAL, "render %d is NULL", k);
            if (!seen.insert(r).second) fail(PS_EINVAL, "render %d appears twice in the batch", k);
            const uint8_t* lt = luts ? luts[k] : nullptr;
            checkFrame(r->rig, srcs[k], r->rig.numImages(), lt, r->rig.numImages(), &dsts[k]);
            rigs.push_back(&r->rig);
            in.push_back({srcs[k], lt, &dsts[k]});
        }
        std::lock_guard<std::mutex> lk(g_planMu);
        auto& plan = g_batchPlans[rigs];
        if (!plan || !plan->matches(rigs)) plan.reset(new ps::Plan(rigs));
        plan->run(in, toStream(stream), true);
    });
}

// ---- primitives -----------------------------------------------------------------
int ps_generate_reproject_map_and_mask(const ps_photo_param* param, int src_w, int src_h, int dst_w, int dst_h,
                                       float* xmap, float* ymap, uint8_t* mask, void* stream)
{
    return guarded([&] {
        if (!param || !xmap || !ymap || !mask) fail(PS_EINVAL, "NULL argument");
        if (src_w <= 0 || src_h <= 0 || dst_w <= 0 || dst_h <= 0) fail(PS_EINVAL, "sizes must be positive");
        if (param->image_type < 0 || param->image_type > 3) fail(PS_EINVAL, "image_type not in 0..3");
        ps::RemapDev rp;
        ps::remapInit(*param, dst_w, dst_h, src_w, src_h, rp);
        ps::DevBuf d(sizeof rp);
        PS_CUDA(cudaMemcpyAsync(d.get(), &rp, sizeof rp, cudaMemcpyHostToDevice, toStream(stream)));
        PS_CUDA(ps::launchGenMap(d.as<ps::RemapDev>(), dst_w, dst_h, xmap, ymap, mask, toStream(stream)));
        PS_CUDA(cudaStreamSynchronize(toStream(stream)));
    });
}

int ps_reproject_to_16s(const ps_image* src, const float* xmap, const float* ymap, long long map_pitch, int dst_w,
                        int dst_h, const uint8_t* lut, int16_t* dst, long long dst_pitch, void* stream)
{
    return guarded([&] {
        if (!src || !xmap || !ymap || !dst) fail(PS_EINVAL, "NULL argument");
        checkImage(src, src->width, src->height, "src", 0);
        if (src->location != PS_MEM_DEVICE) fail(PS_EINVAL, "src must be device memory");
        if (src->width <= 0 || src->height <= 0 || dst_w <= 0 || dst_h <= 0) fail(PS_EINVAL, "empty image");
        if (map_pitch < (long long)dst_w * 4 || (map_pitch & 3)) fail(PS_EINVAL, "bad map pitch");
        if (dst_pitch < (long long)dst_w * 8 || (dst_pitch & 7) || (reinterpret_cast<uintptr_t>(dst) & 7))
            fail(PS_EINVAL, "bad dst pitch / alignment");
        PS_CUDA(ps::launchReprojectTo16S(static_cast<const uint8_t*>(src->data), src->pitch, src->width, src->height,
                                         src->format, xmap, ymap, map_pitch, dst_w, dst_h, lut, dst, dst_pitch,
                                         toStream(stream)));
    });
}

int ps_non_intersecting_masks(const uint8_t* masks, int num, int width, int height, uint8_t* out, void* stream)
{
    return guarded([&] {
        if (!masks || !out) fail(PS_EINVAL, "NULL argument");
        if (num <= 0 || num > PS_MAX_CAMS) fail(PS_EINVAL, "%d masks, 1..%d supported", num, PS_MAX_CAMS);
        if (width <= 0 || height <= 0) fail(PS_EINVAL, "mask size (%d, %d) must be positive", width, height);
        const size_t npx = (size_t)width * height;
        ps::DevBuf uni(npx), dUni(npx * 4), dCam(npx * 4);
        PS_CUDA(ps::launchNonIntersectingMasks(masks, num, width, height, out, uni.as<uint8_t>(), dUni.as<int32_t>(),
                                               dCam.as<int32_t>(), toStream(stream)));
        PS_CUDA(cudaStreamSynchronize(toStream(stream)));
    });
}

int ps_distance_transform_l1(const uint8_t* mask, int width, int height, int32_t* dist, void* stream)
{
    return guarded([&] {
        if (!mask || !dist) fail(PS_EINVAL, "NULL argument");
        if (width <= 0 || height <= 0) fail(PS_EINVAL, "mask size (%d, %d) must be positive", width, height);
        PS_CUDA(ps::launchDistanceTransformL1(mask, width, height, dist, toStream(stream)));
    });
}

int ps_cvt_bgr32_to_yuv(const ps_image* src, const ps_planar_image* dst, void* stream)
{
    return guarded([&] {
        if (!src || !dst) fail(PS_EINVAL, "NULL argument");
        checkImage(src, src->width, src->height, "src", 0);
        if (src->format != PS_FMT_BGR32) fail(PS_EINVAL, "src must be BGR32");  // CV_8UC4, ImageProc.cu:123
        if (src->location != PS_MEM_DEVICE) fail(PS_EINVAL, "src must be device memory");
        checkPlanar(dst, src->width, src->height, "dst");
        if (dst->location != PS_MEM_DEVICE) fail(PS_EINVAL, "dst must be device memory");
        PS_CUDA(ps::launchCvtYuv(static_cast<const uint8_t*>(src->data), src->pitch, src->width, src->height,
                                 dst->format, static_cast<uint8_t*>(dst->planes[0]), dst->pitches[0],
                                 static_cast<uint8_t*>(dst->planes[1]), dst->pitches[1],
                                 static_cast<uint8_t*>(dst->planes[2]), dst->pitches[2], toStream(stream)));
    });
}

int ps_cvt_yuv_to_bgr32(const ps_planar_image* src, const ps_image* dst, void* stream)
{
    return guarded([&] {
        if (!src || !dst) fail(PS_EINVAL, "NULL argument");
        checkPlanar(src, src->width, src->height, "src");
        if (src->location != PS_MEM_DEVICE) fail(PS_EINVAL, "src must be device memory");
        checkImage(dst, src->width, src->height, "dst", 0);
        if (dst->format != PS_FMT_BGR32) fail(PS_EINVAL, "dst must be BGR32");  // CV_8UC4, ImageProc.cu:231
        if (dst->location != PS_MEM_DEVICE) fail(PS_EINVAL, "dst must be device memory");
        ps::YuvFrames f;
        std::memset(&f, 0, sizeof f);
        f.n = 1;
        f.w = src->width;
        f.h = src->height;
        ps::YuvFrame& F = f.frame[0];
        F.fmt = src->format;
        F.y = static_cast<const uint8_t*>(src->planes[0]);
        F.yPitch = src->pitches[0];
        F.u = static_cast<const uint8_t*>(src->planes[1]);
        F.uPitch = src->pitches[1];
        if (src->format == PS_FMT_YUV420P) {
            F.v = static_cast<const uint8_t*>(src->planes[2]);
            F.vPitch = src->pitches[2];
        }
        F.dst = static_cast<uint8_t*>(dst->data);
        F.dstPitch = dst->pitch;
        PS_CUDA(ps::launchYuvToBgr32(f, toStream(stream)));
    });
}

long long ps_debug_bounds_violations(int reset) { return ps::boundsViolations(reset != 0); }

int ps_get_lut(double k, uint8_t* lut256)
{
    return guarded([&] {
        if (!lut256) fail(PS_EINVAL, "lut is NULL");
        if (!(k > 0)) fail(PS_EINVAL, "k = %g must be positive", k);  // CV_Assert(k > 0)
        for (int i = 0; i < 256; i++) {
            const double v = std::nearbyint(k * i);
            lut256[i] = (uint8_t)(v < 0 ? 0 : (v > 255 ? 255 : v));
        }
    });
}

// ---- blender ----------------------------------------------------------------------
int ps_blender_create(ps_blender** out)
{
    return guarded([&] {
        if (!out) fail(PS_EINVAL, "out is NULL");
        *out = new ps_blender();
    });
}

void ps_blender_destroy(ps_blender* b) { delete b; }

int ps_blender_prepare(ps_blender* b, const uint8_t* const* masks, const uint8_t* const* seams, int num, int width,
                       int height, int max_levels, int min_length, void* stream)
{
    return guarded([&] {
        if (!b) fail(PS_EINVAL, "blender is NULL");
        b->plan.reset();
        b->rig.prepareFromMasks(masks, seams, num, width, height, max_levels, min_length, toStream(stream));
        b->plan.reset(new ps::Plan({&b->rig}));
    });
}

int ps_blender_set_custom_masks(ps_blender* b, const uint8_t* const* masks, int num_masks, void* stream)
{
    return guarded([&] {
        if (!b) fail(PS_EINVAL, "blender is NULL");
        setCustomMasks(b->rig, masks, num_masks, stream);
    });
}

int ps_blender_blend(ps_blender* b, const void* const* images, const long long* pitches, int image_format,
                     ps_image* dst, void* stream)
{
    return guarded([&] {
        if (!b) fail(PS_EINVAL, "blender is NULL");
        if (!b->rig.ready()) fail(PS_ESTATE, "have not prepared or prepare failed before");
        if (!images || !pitches) fail(PS_EINVAL, "NULL images");
        if (image_format != 16 && image_format != 8) fail(PS_EINVAL, "image_format %d is neither 16 nor 8", image_format);
        const int esz = image_format == 16 ? 8 : 4;
        for (int i = 0; i < b->rig.numImages(); i++) {
            if (!images[i]) fail(PS_EINVAL, "image %d is NULL", i);
            if (pitches[i] < (long long)b->rig.width() * esz || (pitches[i] % esz) ||
                (reinterpret_cast<uintptr_t>(images[i]) % esz))
                fail(PS_EINVAL, "image %d: bad pitch or alignment", i);
        }
        checkImage(dst, b->rig.width(), b->rig.height(), "dst", 0);
        const int slot = b->rig.peekSlot();  // the state slot the next run takes
        PS_CUDA(cudaStreamWaitEvent(toStream(stream), b->rig.slotComputed(slot), 0));
        b->rig.imagesToLevel0(images, pitches, image_format, slot, toStream(stream));
        if (!b->plan || !b->plan->matches({&b->rig})) b->plan.reset(new ps::Plan({&b->rig}));
        b->plan->run({ps::FrameInput{nullptr, nullptr, dst}}, toStream(stream), false);
    });
}

int ps_blender_get_num_levels(const ps_blender* b) { return b && b->rig.ready() ? b->rig.numLevels() : 0; }

int ps_blender_begin(ps_blender* b, void* stream)
{
    return guarded([&] {
        if (!b) fail(PS_EINVAL, "blender is NULL");
        if (!b->rig.ready()) fail(PS_ESTATE, "have not prepared or prepare failed before");
        b->tileSlot = b->rig.peekSlot();  // the state slot the next run takes
        PS_CUDA(cudaStreamWaitEvent(toStream(stream), b->rig.slotComputed(b->tileSlot), 0));
        b->tiled = 0;
        b->tiling = true;
    });
}

int ps_blender_tile(ps_blender* b, const void* image, long long pitch, int image_format, int index, void* stream)
{
    return guarded([&] {
        if (!b) fail(PS_EINVAL, "blender is NULL");
        if (!b->tiling) fail(PS_ESTATE, "tile without begin");
        if (index < 0 || index >= b->rig.numImages())
            fail(PS_EINVAL, "index %d out of range 0..%d", index, b->rig.numImages() - 1);
        if (b->tiled >> index & 1) fail(PS_EINVAL, "camera %d was already tiled since begin", index);
        if (image_format != 16 && image_format != 8) fail(PS_EINVAL, "image_format %d is neither 16 nor 8", image_format);
        const int esz = image_format == 16 ? 8 : 4;
        if (!image) fail(PS_EINVAL, "image is NULL");
        if (pitch < (long long)b->rig.width() * esz || (pitch % esz) || (reinterpret_cast<uintptr_t>(image) % esz))
            fail(PS_EINVAL, "image: bad pitch or alignment");
        b->rig.imageToLevel0(image, pitch, image_format, index, b->tileSlot, toStream(stream));
        b->tiled |= 1ull << index;
    });
}

int ps_blender_end(ps_blender* b, ps_image* dst, void* stream)
{
    return guarded([&] {
        if (!b) fail(PS_EINVAL, "blender is NULL");
        if (!b->tiling) fail(PS_ESTATE, "end without begin");
        checkImage(dst, b->rig.width(), b->rig.height(), "dst", 0);
        b->tiling = false;
        if (b->rig.peekSlot() != b->tileSlot) fail(PS_ESTATE, "the blender ran another blend since begin");
        for (int i = 0; i < b->rig.numImages(); i++)
            if (!(b->tiled >> i & 1)) b->rig.zeroLevel0(i, b->tileSlot, toStream(stream));
        if (!b->plan || !b->plan->matches({&b->rig})) b->plan.reset(new ps::Plan({&b->rig}));
        b->plan->run({ps::FrameInput{nullptr, nullptr, dst}}, toStream(stream), false);
    });
}

int ps_blender_get_unique_masks(const ps_blender* b, uint8_t* const* masks, int num)
{
    return guarded([&] {
        if (!b) fail(PS_EINVAL, "blender is NULL");
        if (!b->rig.ready()) fail(PS_ESTATE, "have not prepared or prepare failed before");
        if (!masks || num != b->rig.numImages())
            fail(PS_EINVAL, "%d mask buffers given, %d images prepared", num, b->rig.numImages());
        const long long bytes = (long long)b->rig.width() * b->rig.height();
        for (int i = 0; i < num; i++) {
            if (!masks[i]) fail(PS_EINVAL, "mask buffer %d is NULL", i);
            b->rig.exportState(3, i, 0, masks[i], bytes);
        }
    });
}

long long ps_blender_used_memory(const ps_blender* b) { return b && b->rig.ready() ? b->rig.residentBytes() : 0; }

long long ps_blender_estimate_memory(int width, int height, int num_images, int max_levels)
{
    long long v = -1;
    const int st = guarded([&] { v = ps::Rig::estimateBlenderBytes(width, height, num_images, max_levels); });
    return st == PS_OK ? v : -1;
}

int ps_blender_check(ps_blender* b)
{
    return guarded([&] {
        if (!b) fail(PS_EINVAL, "blender is NULL");
        if (!b->rig.ready()) return;
        const int st = b->rig.takeStatus();
        if (st & 4)
            fail(PS_ETIMEOUT, "a bounded wait of a blend kernel ran out: blends since the last check may be wrong");
    });
}

int ps_blender_set_wait_probe(ps_blender* b, int polls)
{
    return guarded([&] {
        if (!b) fail(PS_EINVAL, "blender is NULL");
        if (!b->rig.ready()) fail(PS_ESTATE, "have not prepared or prepare failed before");
        b->rig.setWaitProbe(polls);
    });
}

}  // extern "C"
