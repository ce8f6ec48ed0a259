/*
 * ps_oracle_cpu.c -- CPU restatement of the reference's CPU multiband blend,
 * TilingMultibandBlendFast (source/Blend/MultiBandBlend.cpp:906-1031), with
 * the OpenCV-style pyramids it calls (source/Blend/Pyramid.cpp:35-594), and
 * of the CPU render around it (CPUPanoramaRender::render,
 * source/Task/RicohUtil.cpp:1481-1587).
 *
 * TEST INFRASTRUCTURE ONLY.  The CUDA product computes the CudaAccel
 * semantics (ps_oracle.c restates those).  The reference's CPU twin of the
 * blend differs from them on purpose-free details: its masked pyrDown
 * divides ((S << 8) - S) by the alpha sum (x255, not x256), its full-mask
 * normalisation is R >> 8 without rounding, and its Laplacian subtract
 * saturates.  This file gives that twin for two uses: the secondary
 * difference histogram (product against the CPU semantics) and the timed
 * reference arm (the reference's own CPU path).  It is pinned bit for bit
 * to the reference's TilingMultibandBlendFast compiled in oracle/_ref/
 * (tests/test_ref_pin.py).
 *
 * Threading: the reference builds one camera's pyramid per thread
 * (TilingMultibandBlendFastParallel, :1430-1482).  Here every pass runs
 * row bands of one level on a pool of host threads.  All arithmetic is
 * integer and every output element is written by exactly one thread, so the
 * result does not depend on the thread count.
 */
#include "ps_oracle.h"

#include <pthread.h>
#include <stdatomic.h>
#include <stdlib.h>
#include <string.h>

/* ======================================================================== */
/* A small pool of host threads: parallel for over [0, n) in chunks.         */
/* ======================================================================== */

typedef void (*range_fn)(void* ctx, int lo, int hi);

typedef struct {
    pthread_t* th;
    int nworkers;
    pthread_mutex_t mu;
    pthread_cond_t go, done;
    unsigned gen;
    int quit, finished;
    range_fn fn;
    void* ctx;
    int n, chunk;
    atomic_int next;
} pool_t;

static void pool_run_chunks(pool_t* p)
{
    for (;;) {
        int lo = atomic_fetch_add(&p->next, p->chunk);
        if (lo >= p->n) break;
        int hi = lo + p->chunk < p->n ? lo + p->chunk : p->n;
        p->fn(p->ctx, lo, hi);
    }
}

static void* pool_worker(void* arg)
{
    pool_t* p = (pool_t*)arg;
    unsigned seen = 0;
    for (;;) {
        pthread_mutex_lock(&p->mu);
        while (p->gen == seen && !p->quit) pthread_cond_wait(&p->go, &p->mu);
        if (p->quit) {
            pthread_mutex_unlock(&p->mu);
            return NULL;
        }
        seen = p->gen;
        pthread_mutex_unlock(&p->mu);
        pool_run_chunks(p);
        pthread_mutex_lock(&p->mu);
        if (++p->finished == p->nworkers) pthread_cond_signal(&p->done);
        pthread_mutex_unlock(&p->mu);
    }
}

static pool_t* pool_create(int nthreads)
{
    pool_t* p = (pool_t*)calloc(1, sizeof(pool_t));
    p->nworkers = nthreads > 1 ? nthreads - 1 : 0;  /* the caller is the last worker */
    pthread_mutex_init(&p->mu, NULL);
    pthread_cond_init(&p->go, NULL);
    pthread_cond_init(&p->done, NULL);
    p->th = (pthread_t*)calloc(p->nworkers ? (size_t)p->nworkers : 1, sizeof(pthread_t));
    for (int t = 0; t < p->nworkers; t++) pthread_create(&p->th[t], NULL, pool_worker, p);
    return p;
}

static void pool_for(pool_t* p, int n, int chunk, range_fn fn, void* ctx)
{
    if (n <= 0) return;
    if (chunk < 1) chunk = 1;
    if (p->nworkers == 0 || n <= chunk) {
        fn(ctx, 0, n);
        return;
    }
    pthread_mutex_lock(&p->mu);
    p->fn = fn;
    p->ctx = ctx;
    p->n = n;
    p->chunk = chunk;
    atomic_store(&p->next, 0);
    p->finished = 0;
    p->gen++;
    pthread_cond_broadcast(&p->go);
    pthread_mutex_unlock(&p->mu);
    pool_run_chunks(p);
    pthread_mutex_lock(&p->mu);
    while (p->finished < p->nworkers) pthread_cond_wait(&p->done, &p->mu);
    pthread_mutex_unlock(&p->mu);
}

static void pool_destroy(pool_t* p)
{
    pthread_mutex_lock(&p->mu);
    p->quit = 1;
    pthread_cond_broadcast(&p->go);
    pthread_mutex_unlock(&p->mu);
    for (int t = 0; t < p->nworkers; t++) pthread_join(p->th[t], NULL);
    pthread_mutex_destroy(&p->mu);
    pthread_cond_destroy(&p->go);
    pthread_cond_destroy(&p->done);
    free(p->th);
    free(p);
}

/* Row chunk that keeps a pass to a few dozen pool grabs per thread. */
static int row_chunk(int rows, int nthreads) { int c = rows / (8 * (nthreads > 0 ? nthreads : 1)); return c < 1 ? 1 : c; }

/* ======================================================================== */
/* Borders: OpenCV's borderInterpolate for the two kinds the CPU pyramids    */
/* use -- BORDER_WRAP horizontally, BORDER_DEFAULT (reflect-101) vertically. */
/* ======================================================================== */

static inline int wrap_index(int p, int len)
{
    if (p >= 0 && p < len) return p;
    p %= len;
    return p < 0 ? p + len : p;
}

/* Reflect-101 (mirror about the edge pixel, which is not repeated); every
   index maps to 0 when len == 1. */
static inline int reflect101_index(int p, int len)
{
    if (p >= 0 && p < len) return p;
    if (len == 1) return 0;
    while (p < 0 || p >= len) p = p < 0 ? -p : 2 * len - 2 - p;
    return p;
}

/* ======================================================================== */
/* The blender                                                               */
/* ======================================================================== */

struct orc_cpu_blender {
    int n, W, H, L, full;
    int ws[17], hs[17];
    size_t off[18];   /* pixel offset of each level in a packed pyramid */
    int16_t* weight;  /* n * total: weightPyrs (int16, one channel) */
    int32_t* alpha;   /* n * total: alphaPyrs (levels >= 1; level 0 unused) */
    int32_t* wsum;    /* total: resultWeightPyr (only if !full) */
    uint8_t* masknot; /* W*H: maskNot (only if !full) */
    /* Working memory, allocated once and reused by every blend, as the
       reference allocates its pyramids at prepare (:929-930): returning it
       to the system after each frame makes every frame fault it in again,
       which costs far more than the blend on hosts that keep device page
       tables coherent with the CPU's. */
    int16_t* g;       /* 3 * total: one camera's image pyramid (imagePyr) */
    int32_t* res;     /* 3 * total: resultPyr */
    int16_t* level0;  /* n * W*H*4: the render's remapped images */
    uint8_t* lutted;  /* the render's LUT'd source frame */
    size_t luttedBytes;
    pool_t* pool;
    int poolThreads;
};

static pool_t* blender_pool(orc_cpu_blender* b, int nthreads)
{
    if (!b->pool || b->poolThreads != nthreads) {
        if (b->pool) pool_destroy(b->pool);
        b->pool = pool_create(nthreads);
        b->poolThreads = nthreads;
    }
    return b->pool;
}

static size_t cpu_total(const orc_cpu_blender* b) { return b->off[b->L + 1]; }

/* ---- pyrDown (pyrDown_, source/Blend/Pyramid.cpp:35-149,304-411) ------------
   Output pixel (x, y) of a level is the 5x5 sum, weights 1 4 6 4 1 in each
   direction, of the input at columns wrap(2x-2 .. 2x+2) and rows
   reflect101(2y-2 .. 2y+2).  The pyramidDownTo32S form keeps the raw sum;
   pyramidDown of int16 rounds it as (S + 128) >> 8 (FixPtCast<short, 8>). */
static const int K5[5] = {1, 4, 6, 4, 1};

static inline int down_sum_1(const int16_t* src, int sw, int sh, int x, int y)
{
    int s = 0;
    for (int ky = 0; ky < 5; ky++) {
        const int16_t* row = src + (size_t)reflect101_index(2 * y + ky - 2, sh) * sw;
        int h = 0;
        for (int kx = 0; kx < 5; kx++) h += K5[kx] * row[wrap_index(2 * x + kx - 2, sw)];
        s += K5[ky] * h;
    }
    return s;
}

/* ---- prepare (TilingMultibandBlendFast::prepare, MultiBandBlend.cpp:906-985) */
orc_cpu_blender* orc_cpu_mb_prepare(const uint8_t* masks, const uint8_t* seams, int n, int W, int H, int maxLevels,
                                    int minLength)
{
    if (n <= 0 || n > 255 || W <= 0 || H <= 0) return NULL;
    orc_cpu_blender* b = (orc_cpu_blender*)calloc(1, sizeof(orc_cpu_blender));
    b->n = n;
    b->W = W;
    b->H = H;
    b->L = orc_num_levels(W, H, maxLevels, minLength);                  /* :927 */
    orc_level_sizes(W, H, b->L, b->ws, b->hs);                           /* :929-930 */
    b->off[0] = 0;
    for (int j = 0; j <= b->L; j++) b->off[j + 1] = b->off[j] + (size_t)b->ws[j] * b->hs[j];
    const size_t tot = cpu_total(b), npx = (size_t)W * H;
    b->g = (int16_t*)malloc(sizeof(int16_t) * 3 * tot);
    b->res = (int32_t*)malloc(sizeof(int32_t) * 3 * tot);
    b->weight = (int16_t*)calloc((size_t)n * tot, sizeof(int16_t));
    b->alpha = (int32_t*)calloc((size_t)n * tot, sizeof(int32_t));
    int16_t* tmp = (int16_t*)malloc(sizeof(int16_t) * tot);
    for (int i = 0; i < n; i++) {
        /* weightPyrs: createGaussPyramid of 256 on the unique mask (:936-942) */
        int16_t* wt = b->weight + (size_t)i * tot;
        for (size_t p = 0; p < npx; p++) wt[p] = seams[(size_t)i * npx + p] ? 256 : 0;
        for (int j = 0; j < b->L; j++)
            for (int y = 0; y < b->hs[j + 1]; y++)
                for (int x = 0; x < b->ws[j + 1]; x++)
                    wt[b->off[j + 1] + (size_t)y * b->ws[j + 1] + x] =
                        (int16_t)((down_sum_1(wt + b->off[j], b->ws[j], b->hs[j], x, y) + 128) >> 8);
        /* alphaPyrs: pyramidDownTo32S of 256 on the coverage, the next level's
           input 256 wherever that sum is non-zero (:944-957,
           setAlpha16SAccordingToAlpha32S :714-730) */
        int32_t* al = b->alpha + (size_t)i * tot;
        for (size_t p = 0; p < npx; p++) tmp[p] = masks[(size_t)i * npx + p] ? 256 : 0;
        for (int j = 0; j < b->L; j++) {
            for (int y = 0; y < b->hs[j + 1]; y++)
                for (int x = 0; x < b->ws[j + 1]; x++) {
                    const size_t o = b->off[j + 1] + (size_t)y * b->ws[j + 1] + x;
                    al[o] = down_sum_1(tmp + b->off[j], b->ws[j], b->hs[j], x, y);
                    tmp[o] = al[o] ? 256 : 0;
                }
        }
    }
    free(tmp);
    /* fullMask, resultWeightPyr, maskNot (:959-982) */
    size_t covered = 0;
    uint8_t* uni = (uint8_t*)calloc(npx, 1);
    for (size_t p = 0; p < npx; p++) {
        for (int i = 0; i < n; i++)
            if (masks[(size_t)i * npx + p]) { uni[p] = 1; break; }
        covered += uni[p];
    }
    b->full = covered == npx;
    if (!b->full) {
        b->wsum = (int32_t*)calloc(tot, sizeof(int32_t));
        for (int i = 0; i < n; i++) {
            const int16_t* wt = b->weight + (size_t)i * tot;
            for (size_t p = 0; p < tot; p++) b->wsum[p] += wt[p];
        }
        b->masknot = (uint8_t*)malloc(npx);
        for (size_t p = 0; p < npx; p++) b->masknot[p] = uni[p] ? 0 : 255;
    }
    free(uni);
    return b;
}

void orc_cpu_mb_free(orc_cpu_blender* b)
{
    if (!b) return;
    free(b->weight);
    free(b->alpha);
    free(b->wsum);
    free(b->masknot);
    free(b->g);
    free(b->res);
    free(b->level0);
    free(b->lutted);
    if (b->pool) pool_destroy(b->pool);
    free(b);
}

int orc_cpu_mb_num_levels(const orc_cpu_blender* b) { return b->L; }
int orc_cpu_mb_full_mask(const orc_cpu_blender* b) { return b->full; }

void orc_cpu_mb_get_weight(const orc_cpu_blender* b, int cam, int level, int16_t* out)
{
    memcpy(out, b->weight + (size_t)cam * cpu_total(b) + b->off[level],
           sizeof(int16_t) * (size_t)b->ws[level] * b->hs[level]);
}

void orc_cpu_mb_get_alpha(const orc_cpu_blender* b, int cam, int level, int32_t* out)
{
    memcpy(out, b->alpha + (size_t)cam * cpu_total(b) + b->off[level],
           sizeof(int32_t) * (size_t)b->ws[level] * b->hs[level]);
}

/* ---- blend (TilingMultibandBlendFast::blend, MultiBandBlend.cpp:987-1031) ---- */
typedef struct {
    const orc_cpu_blender* b;
    int cam, j;
    int16_t* g;          /* the camera's int16x3 pyramid, packed (3 per pixel) */
    int32_t* res;        /* resultPyr, int32x3, packed */
    const int16_t* img;  /* level-0 input, int16x4 */
    uint8_t* dst;        /* BGR32 output */
} blend_ctx;

/* level 0 of the camera's pyramid: the image's B, G, R (imagePyr[0] = images[i]) */
static void pass_load(void* arg, int y0, int y1)
{
    blend_ctx* c = (blend_ctx*)arg;
    const int W = c->b->W;
    for (int y = y0; y < y1; y++)
        for (int x = 0; x < W; x++) {
            const size_t p = (size_t)y * W + x;
            for (int ch = 0; ch < 3; ch++) c->g[3 * p + ch] = c->img[4 * p + ch];
        }
}

/* imagePyr[j+1] from imagePyr[j]: pyramidDownTo32S, then calcDstImage
   (:732-768): ((S << 8) - S) / alpha where the alpha sum is non-zero, else 0
   (C division, truncating). */
static void pass_down(void* arg, int y0, int y1)
{
    blend_ctx* c = (blend_ctx*)arg;
    const orc_cpu_blender* b = c->b;
    const int j = c->j, sw = b->ws[j], sh = b->hs[j], dw = b->ws[j + 1];
    const int16_t* src = c->g + 3 * b->off[j];
    int16_t* dst = c->g + 3 * b->off[j + 1];
    const int32_t* al = b->alpha + (size_t)c->cam * cpu_total(b) + b->off[j + 1];
    for (int y = y0; y < y1; y++) {
        const int16_t* rows[5];
        for (int ky = 0; ky < 5; ky++) rows[ky] = src + 3 * (size_t)reflect101_index(2 * y + ky - 2, sh) * sw;
        for (int x = 0; x < dw; x++) {
            int cols[5];
            for (int kx = 0; kx < 5; kx++) cols[kx] = 3 * wrap_index(2 * x + kx - 2, sw);
            const int a = al[(size_t)y * dw + x];
            int16_t* o = dst + 3 * ((size_t)y * dw + x);
            for (int ch = 0; ch < 3; ch++) {
                int s = 0;
                for (int ky = 0; ky < 5; ky++) {
                    int h = 0;
                    for (int kx = 0; kx < 5; kx++) h += K5[kx] * rows[ky][cols[kx] + ch];
                    s += K5[ky] * h;
                }
                o[ch] = a ? (int16_t)(((s << 8) - s) / a) : 0;
            }
        }
    }
}

/* ---- pyrUp (pyrUp_, source/Blend/Pyramid.cpp:413-520) ----------------------
   From a level of sw x sh to dw x dh (dw = 2 sw or 2 sw - 1, likewise dh).
   Horizontally, source column x gives output 2x the sum s[x-1] + 6 s[x] +
   s[x+1] and output 2x+1 the sum 4 (s[x] + s[x+1]), columns wrapped.
   Vertically, with h(r) those row sums of source row reflect101(r):
   output row 2y = h(y-1) + 6 h(y) + h(y+1), output row 2y+1 = 4 (h(y) +
   h(y+1)); each value is then (v + 32) >> 6. */
static inline void up_hrow(const int16_t* row, int sw, int dw, int ch, int* out)
{
    for (int x = 0; x < sw; x++) {
        const int l = row[3 * wrap_index(x - 1, sw) + ch], m = row[3 * x + ch], r = row[3 * wrap_index(x + 1, sw) + ch];
        out[2 * x] = l + m * 6 + r;
        if (2 * x + 1 < dw) out[2 * x + 1] = (m + r) * 4;
    }
}

static inline void up_hrow32(const int32_t* row, int sw, int dw, int ch, int* out)
{
    for (int x = 0; x < sw; x++) {
        const int l = row[3 * wrap_index(x - 1, sw) + ch], m = row[3 * x + ch], r = row[3 * wrap_index(x + 1, sw) + ch];
        out[2 * x] = l + m * 6 + r;
        if (2 * x + 1 < dw) out[2 * x + 1] = (m + r) * 4;
    }
}

/* Laplacian of level j (pyramidUp of imagePyr[j+1], cv::subtract, :1013-1019)
   and its accumulation (accumulate, :106-129: resultPyr += lap * weight).
   Rows y0..y1 are source rows of level j+1. */
static void pass_up_lap(void* arg, int y0, int y1)
{
    blend_ctx* c = (blend_ctx*)arg;
    const orc_cpu_blender* b = c->b;
    const int j = c->j, sw = b->ws[j + 1], sh = b->hs[j + 1], dw = b->ws[j], dh = b->hs[j];
    const int16_t* src = c->g + 3 * b->off[j + 1];
    int16_t* lev = c->g + 3 * b->off[j];
    int32_t* res = c->res + 3 * b->off[j];
    const int16_t* wt = b->weight + (size_t)c->cam * cpu_total(b) + b->off[j];
    int* h = (int*)malloc(sizeof(int) * 3 * (size_t)(dw + 1));
    for (int y = y0; y < y1; y++) {
        int* h0 = h;
        int* h1 = h + (dw + 1);
        int* h2 = h + 2 * (dw + 1);
        for (int ch = 0; ch < 3; ch++) {
            up_hrow(src + 3 * (size_t)reflect101_index(y - 1, sh) * sw, sw, dw, ch, h0);
            up_hrow(src + 3 * (size_t)reflect101_index(y, sh) * sw, sw, dw, ch, h1);
            up_hrow(src + 3 * (size_t)reflect101_index(y + 1, sh) * sw, sw, dw, ch, h2);
            for (int r = 0; r < 2; r++) {
                const int oy = 2 * y + r;
                if (oy >= dh) break;
                for (int x = 0; x < dw; x++) {
                    const int v = r == 0 ? h0[x] + h1[x] * 6 + h2[x] : (h1[x] + h2[x]) * 4;
                    const int up = (int16_t)((v + 32) >> 6);
                    const size_t p = (size_t)oy * dw + x;
                    int d = lev[3 * p + ch] - up;
                    d = d < -32768 ? -32768 : (d > 32767 ? 32767 : d);
                    lev[3 * p + ch] = (int16_t)d;
                    res[3 * p + ch] += d * wt[p];
                }
            }
        }
    }
    free(h);
}

/* resultPyr[i].setTo(0) (:999-1000), over the packed pixels of all levels */
static void pass_zero(void* arg, int p0, int p1)
{
    blend_ctx* c = (blend_ctx*)arg;
    memset(c->res + 3 * (size_t)p0, 0, sizeof(int32_t) * 3 * (size_t)(p1 - p0));
}

/* the top level, a Gaussian, accumulated as it is */
static void pass_top(void* arg, int y0, int y1)
{
    blend_ctx* c = (blend_ctx*)arg;
    const orc_cpu_blender* b = c->b;
    const int L = b->L, w = b->ws[L];
    const int16_t* g = c->g + 3 * b->off[L];
    int32_t* res = c->res + 3 * b->off[L];
    const int16_t* wt = b->weight + (size_t)c->cam * cpu_total(b) + b->off[L];
    for (size_t p = (size_t)y0 * w; p < (size_t)y1 * w; p++)
        for (int ch = 0; ch < 3; ch++) res[3 * p + ch] += g[3 * p + ch] * wt[p];
}

/* normalize(resultPyr) when fullMask: R >> 8 (:141-154); else
   normalize(resultPyr, resultWeightPyr): R / w, with w = 0 taken as 1
   (:213-240).  Over the packed pixels of all levels. */
static void pass_norm(void* arg, int p0, int p1)
{
    blend_ctx* c = (blend_ctx*)arg;
    const orc_cpu_blender* b = c->b;
    for (size_t p = (size_t)p0; p < (size_t)p1; p++) {
        int32_t* r = c->res + 3 * p;
        if (b->full) {
            for (int ch = 0; ch < 3; ch++) r[ch] >>= 8;
        } else {
            int w = b->wsum[p];
            if (!w) w++;
            for (int ch = 0; ch < 3; ch++) r[ch] /= w;
        }
    }
}

/* restoreImageFromLaplacePyramid (:770-781): resultPyr[j] += pyramidUp of
   resultPyr[j+1] (int32, (v + 32) >> 6).  Rows are source rows of level j+1. */
static void pass_collapse(void* arg, int y0, int y1)
{
    blend_ctx* c = (blend_ctx*)arg;
    const orc_cpu_blender* b = c->b;
    const int j = c->j, sw = b->ws[j + 1], sh = b->hs[j + 1], dw = b->ws[j], dh = b->hs[j];
    const int32_t* src = c->res + 3 * b->off[j + 1];
    int32_t* lev = c->res + 3 * b->off[j];
    int* h = (int*)malloc(sizeof(int) * 3 * (size_t)(dw + 1));
    for (int y = y0; y < y1; y++) {
        int* h0 = h;
        int* h1 = h + (dw + 1);
        int* h2 = h + 2 * (dw + 1);
        for (int ch = 0; ch < 3; ch++) {
            up_hrow32(src + 3 * (size_t)reflect101_index(y - 1, sh) * sw, sw, dw, ch, h0);
            up_hrow32(src + 3 * (size_t)reflect101_index(y, sh) * sw, sw, dw, ch, h1);
            up_hrow32(src + 3 * (size_t)reflect101_index(y + 1, sh) * sw, sw, dw, ch, h2);
            for (int r = 0; r < 2; r++) {
                const int oy = 2 * y + r;
                if (oy >= dh) break;
                for (int x = 0; x < dw; x++) {
                    const int v = r == 0 ? h0[x] + h1[x] * 6 + h2[x] : (h1[x] + h2[x]) * 4;
                    lev[3 * ((size_t)oy * dw + x) + ch] += (v + 32) >> 6;
                }
            }
        }
    }
    free(h);
}

/* resultPyr[0].convertTo(blendImage, CV_8U) (saturating), then
   blendImage.setTo(0, maskNot) unless fullMask (:1026-1030). */
static void pass_out(void* arg, int y0, int y1)
{
    blend_ctx* c = (blend_ctx*)arg;
    const orc_cpu_blender* b = c->b;
    for (size_t p = (size_t)y0 * b->W; p < (size_t)y1 * b->W; p++) {
        uint8_t* o = c->dst + 4 * p;
        const int keep = b->full || !b->masknot[p];
        for (int ch = 0; ch < 3; ch++) {
            const int v = c->res[3 * p + ch];
            o[ch] = keep ? (uint8_t)(v < 0 ? 0 : (v > 255 ? 255 : v)) : 0;
        }
        o[3] = 0;
    }
}

static void cpu_blend_pool(orc_cpu_blender* b, const int16_t* const* images, uint8_t* dst, int32_t* coll_out,
                           pool_t* pool, int nthreads)
{
    const size_t tot = cpu_total(b);
    blend_ctx c;
    memset(&c, 0, sizeof(c));
    c.b = b;
    c.g = b->g;
    c.res = b->res;
    c.dst = dst;
    const int chunkPx = (int)(tot / (8 * (size_t)nthreads) + 1);
    pool_for(pool, (int)tot, chunkPx, pass_zero, &c);
    const int L = b->L;
    for (int i = 0; i < b->n; i++) {
        c.cam = i;
        c.img = images[i];
        pool_for(pool, b->H, row_chunk(b->H, nthreads), pass_load, &c);
        for (int j = 0; j < L; j++) {  /* :1008-1012 */
            c.j = j;
            pool_for(pool, b->hs[j + 1], row_chunk(b->hs[j + 1], nthreads), pass_down, &c);
        }
        for (int j = 0; j < L; j++) {  /* :1013-1017, accumulate :1018 */
            c.j = j;
            pool_for(pool, b->hs[j + 1], row_chunk(b->hs[j + 1], nthreads), pass_up_lap, &c);
        }
        pool_for(pool, b->hs[L], row_chunk(b->hs[L], nthreads), pass_top, &c);
    }
    pool_for(pool, (int)tot, chunkPx, pass_norm, &c);  /* :1021-1024 */
    for (int j = L - 1; j >= 0; j--) {  /* :1025 */
        c.j = j;
        pool_for(pool, b->hs[j + 1], row_chunk(b->hs[j + 1], nthreads), pass_collapse, &c);
    }
    if (coll_out) memcpy(coll_out, c.res, sizeof(int32_t) * 3 * tot);
    pool_for(pool, b->H, row_chunk(b->H, nthreads), pass_out, &c);
}

void orc_cpu_mb_blend(orc_cpu_blender* b, const int16_t* const* images, uint8_t* dst, int32_t* coll_out,
                      int nthreads)
{
    if (nthreads < 1) nthreads = 1;
    cpu_blend_pool(b, images, dst, coll_out, blender_pool(b, nthreads), nthreads);
}

/* ======================================================================== */
/* The CPU render: per camera the LUT (transform, RicohUtil.cpp:1564-1569),  */
/* the row-parallel bilinear remap to int16 (reprojectParallelTo16S,         */
/* source/Warp/ZReproject.cpp:535-567), then the blend (:1570).              */
/* ======================================================================== */

typedef struct {
    const uint8_t* src;
    const uint8_t* lut;
    uint8_t* lutted;
    int srcW, srcH, channels, dstW;
    const float *xmap, *ymap;
    int16_t* dst;
} render_ctx;

static void pass_lut(void* arg, int y0, int y1)
{
    render_ctx* c = (render_ctx*)arg;
    const size_t rowBytes = (size_t)c->srcW * c->channels;
    for (int y = y0; y < y1; y++) {
        const uint8_t* s = c->src + (size_t)y * rowBytes;
        uint8_t* o = c->lutted + (size_t)y * rowBytes;
        for (int x = 0; x < c->srcW; x++) {
            for (int ch = 0; ch < 3; ch++) o[x * c->channels + ch] = c->lut[ch * 256 + s[x * c->channels + ch]];
            if (c->channels == 4) o[x * c->channels + 3] = 0;
        }
    }
}

static void pass_remap(void* arg, int y0, int y1)
{
    render_ctx* c = (render_ctx*)arg;
    orc_reproject_bilinear_16s_rows(c->lut ? c->lutted : c->src, c->srcW, c->srcH, (long long)c->srcW * c->channels,
                                    c->channels, NULL, c->xmap, c->ymap, c->dstW, y0, y1, c->dst);
}

void orc_cpu_render(orc_cpu_blender* b, const uint8_t* const* srcs, int srcW, int srcH, int channels,
                    const uint8_t* luts, const float* const* xmaps, const float* const* ymaps, uint8_t* dst,
                    int nthreads)
{
    if (nthreads < 1) nthreads = 1;
    pool_t* pool = blender_pool(b, nthreads);
    const size_t npx = (size_t)b->W * b->H;
    if (!b->level0) b->level0 = (int16_t*)malloc(sizeof(int16_t) * 4 * npx * (size_t)b->n);
    const size_t lb = (size_t)srcW * srcH * channels;
    if (luts && b->luttedBytes < lb) {
        free(b->lutted);
        b->lutted = (uint8_t*)malloc(lb);
        b->luttedBytes = lb;
    }
    int16_t** imgs = (int16_t**)calloc((size_t)b->n, sizeof(int16_t*));
    render_ctx c;
    memset(&c, 0, sizeof(c));
    c.lutted = b->lutted;
    for (int i = 0; i < b->n; i++) {
        imgs[i] = b->level0 + 4 * npx * (size_t)i;
        c.src = srcs[i];
        c.lut = luts ? luts + (size_t)i * 768 : NULL;
        c.srcW = srcW;
        c.srcH = srcH;
        c.channels = channels;
        c.dstW = b->W;
        c.xmap = xmaps[i];
        c.ymap = ymaps[i];
        c.dst = imgs[i];
        if (c.lut) pool_for(pool, srcH, row_chunk(srcH, nthreads), pass_lut, &c);
        pool_for(pool, b->H, row_chunk(b->H, nthreads), pass_remap, &c);
    }
    cpu_blend_pool(b, (const int16_t* const*)imgs, dst, NULL, pool, nthreads);
    free(imgs);
}
