// Host side of the C ABI declared in include/cos_capon.h.
//
// The context plays the role of the reference's Capon object
// (RealTimeCapon/Capon.h:13-125): it caches device buffers that grow on demand
// (Capon.cpp:110-148, 465-547) and returns CUDA error numbers as status.
// Unlike the reference it runs every stage on one stream without host
// synchronisation between stages, and keeps covariance matrices on chip.
#include <cuda_runtime.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <algorithm>
#include <map>
#include <new>
#include <tuple>
#include <vector>

#include "capon_internal.h"
#include "../../include/cos_capon.h"

using namespace cgb;

struct DevBuf {
    void *p = nullptr;
    size_t cap = 0;
    int ensure(size_t bytes)
    {
        if (bytes <= cap) return 0;
        if (p) cudaFree(p);
        p = nullptr;
        cap = 0;
        if (cudaMalloc(&p, bytes) != cudaSuccess) {
            cudaGetLastError();
            return COS_CAPON_ERR_OUT_OF_MEMORY;
        }
        cap = bytes;
        return 0;
    }
    void release()
    {
        if (p) cudaFree(p);
        p = nullptr;
        cap = 0;
    }
};

struct cos_capon_ctx {
    int device = 0;
    int num_sms = 0;
    cudaStream_t stream = nullptr;
    unsigned *d_status = nullptr;
    // host-pointer call buffers
    DevBuf x, z, P, w, R;
    // plain / precise pipeline scratch
    DevBuf Rwork, Rlo, dl, Ria;
    // float-float covariance slots of the fused refinement mode (L > 32)
    DevBuf stash;
    // stage entry points
    DevBuf A, b, sol;
    DevBuf V;           // subspace matrix of the host-pointer subspace call
    DevBuf tdib_in;     // inputs of the host-pointer steering call
    DevBuf lca_pw;      // |Z|^2 planes of the LCA selection
    // autotuner: chosen fused candidate per (L, K, M, FusedMode)
    std::map<std::tuple<int, int, int, int>, int> tuned;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    // second stream of the pipelined host-pointer call
    cudaStream_t stream2 = nullptr;
    // auxiliary streams of a multi-frame call: launch groups that use no
    // context scratch run concurrently, forked from and joined back to the
    // caller's stream by events (parallel branches when the call is captured)
    static constexpr int kAux = 3;
    cudaStream_t aux[kAux] = {};
    cudaEvent_t fork_ev = nullptr, join_ev[kAux] = {};
};

static const cos_capon_opts kDefaultOpts = {COS_CAPON_FORM_FUSED, COS_CAPON_LOAD_ELEMENT, COS_CAPON_R_REFERENCE, 0, 0,
                                            0};

// Argument checks of Capon::getCapon (Capon.cpp:98-107) and BuildR::getR
// (BuildR.cpp:37-48), plus this build's own limits.
static int check_sizes(int L, int K, int M, int Nx, int Ny, int Nb)
{
    if (Nx < 1 || Ny < 1 || L < 1 || M < 1 || K < 0 || Nb < 0) return COS_CAPON_ERR_LAUNCH;
    if (Nb > L) return COS_CAPON_ERR_LAUNCH;
    if (L > M) return COS_CAPON_ERR_LAUNCH;
    if (2 * K >= Ny) return COS_CAPON_ERR_LAUNCH;
    if (L > 64) return COS_CAPON_ERR_NOT_SUPPORTED;
    return 0;
}

// Reference behaviour: refuse a problem that does not fit in free device memory
// (largerThanMaxSupportedSize, Capon.cpp:549-567).
static int check_free(size_t need)
{
    size_t fr = 0, tot = 0;
    if (cudaMemGetInfo(&fr, &tot) != cudaSuccess) {
        cudaGetLastError();
        return COS_CAPON_ERR_OUT_OF_MEMORY;
    }
    return need > fr ? COS_CAPON_ERR_OUT_OF_MEMORY : 0;
}

static FrameDev make_frame(const cos_capon_frame &fr, const cos_capon_opts &o)
{
    FrameDev f;
    memset(&f, 0, sizeof(f));
    f.x = (const float2 *)fr.x;
    f.z = (float2 *)fr.z;
    f.P = fr.P;
    f.w = (float2 *)fr.w;
    f.R = (float2 *)fr.R;
    f.d = fr.d;
    f.L = fr.L;
    f.K = fr.K;
    f.M = fr.M;
    f.Nx = fr.Nx;
    f.Ny = fr.Ny;
    f.Nb = fr.Nb;
    f.V = fr.Nb > 0 ? (const float2 *)fr.V : nullptr;
    f.Npy = fr.Ny - 2 * fr.K;
    f.loading = o.loading;
    f.r_layout = o.r_layout;
    f.refine = o.refine;
    f.fb = o.fb ? 1 : 0;
    if (o.form == COS_CAPON_FORM_SLIDING_INVERSE) f.tile = o.segment;
    return f;
}

static int candidates(int L, int K, int form, const FusedCandidate **out)
{
    *out = nullptr;
    if (form == COS_CAPON_FORM_TC_FUSED) return tc_fused_candidates(out);
    const int T = 2 * K + 1;
    if (L == 16 && T == 1) return fused_candidates_l16_t1(out);
    if (L == 16 && T == 3) return fused_candidates_l16_t3(out);
    if (L == 16 && T == 5) return fused_candidates_l16_t5(out);
    if (L == 32 && T == 1) return fused_candidates_l32_t1(out);
    if (L == 32 && T == 3) return fused_candidates_l32_t3(out);
    if (L == 32 && T == 5) return fused_candidates_l32_t5(out);
    if (L == 48) return fused_candidates_l48(out);
    if (L == 64) return fused_candidates_l64(out);
    return 0;
}

// a candidate serves a frame when its compile-time L, T (0: any) and M (0: any)
// match and it has the mode: the refinement modes where it carries a stash,
// the others where it is not a refinement-only instantiation
static bool cand_fits(const FusedCandidate &c, const FrameDev &f, bool refining)
{
    if (refining ? !c.stash : c.refine_only) return false;
    return c.L == f.L && (c.T == 0 || c.T == 2 * f.K + 1) && (c.M == 0 || c.M == f.M) &&
           c.smem(f.K, f.M) <= kFusedSmemMax;
}
static bool refining_mode(int mode) { return mode > FUSED_R; }

// the fused path carries the refinement step itself (the blocked per-pixel
// path, instantiated for the refinement modes next to the L = 16 and 32
// kernels); shapes without a fused kernel refine in the precise pipeline
static bool refine_in_fused(const FrameDev &, const cos_capon_opts &o)
{
    return o.form == COS_CAPON_FORM_FUSED;
}

static bool use_fused(const FrameDev &f, const cos_capon_opts &o)
{
    if ((o.form != COS_CAPON_FORM_FUSED && o.form != COS_CAPON_FORM_TC_FUSED) || f.Nb != 0 || o.fb) return false;
    if (o.refine && !refine_in_fused(f, o)) return false;
    const FusedCandidate *c = nullptr;
    const int n = candidates(f.L, f.K, o.form, &c);
    bool refine_fit = false, basic_fit = false;
    for (int i = 0; i < n; ++i) {
        refine_fit |= cand_fits(c[i], f, true);
        basic_fit |= cand_fits(c[i], f, false);
    }
    // with refinement, R (when asked for) still comes from a z/P-w-R candidate
    return o.refine ? refine_fit && (!f.R || basic_fit) : basic_fit;
}

// Autotuner: the first launch of an (L, K, M, mode) shape on a context times
// every candidate configuration on the frames themselves (each candidate
// computes the same per-pixel arithmetic), keeps the fastest, and reruns it so
// that the outputs are the winner's.  COS_CAPON_FUSED_CONFIG=<name> forces a
// candidate.  While the stream is being captured into a graph no timing is
// possible, so an untuned shape then takes the first candidate.
static int launch_fused_tuned(cos_capon_ctx *c, const FramesParam &fp, int mode, int form, cudaStream_t s)
{
    const FrameDev &f0 = fp.f[0];
    const FusedCandidate *cand = nullptr;
    const int n = candidates(f0.L, f0.K, form, &cand);
    std::vector<int> ok;
    for (int i = 0; i < n; ++i) {
        bool fits = true;
        for (int q = 0; q < fp.n; ++q) fits &= cand_fits(cand[i], fp.f[q], refining_mode(mode));
        if (fits) ok.push_back(i);
    }
    if (ok.empty()) return COS_CAPON_ERR_NOT_SUPPORTED;
    if (const char *force = getenv("COS_CAPON_FUSED_CONFIG")) {
        for (int i : ok)
            if (!strcmp(force, cand[i].name)) return cand[i].launch(fp, mode, c->d_status, c->num_sms, s);
    }
    const auto key = std::make_tuple(f0.L, f0.K, f0.M, mode | (form << 8));
    auto it = c->tuned.find(key);
    if (it != c->tuned.end()) return cand[it->second].launch(fp, mode, c->d_status, c->num_sms, s);
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    if (cudaStreamIsCapturing(s, &cs) != cudaSuccess || cs != cudaStreamCaptureStatusNone || ok.size() == 1)
        return cand[ok[0]].launch(fp, mode, c->d_status, c->num_sms, s);
    if (!c->ev0) {
        if (cudaEventCreate(&c->ev0) != cudaSuccess || cudaEventCreate(&c->ev1) != cudaSuccess) {
            cudaGetLastError();
            return cand[ok[0]].launch(fp, mode, c->d_status, c->num_sms, s);
        }
    }
    int best = ok[0];
    float best_ms = 1e30f;
    for (int i : ok) {
        // one untimed launch, then the best of two timed ones
        int e = cand[i].launch(fp, mode, c->d_status, c->num_sms, s);
        if (e == cudaErrorNotSupported) {
            cudaGetLastError();
            continue;
        }
        if (e) return e;
        float ms = 1e30f;
        for (int rep = 0; rep < 2; ++rep) {
            cudaEventRecord(c->ev0, s);
            if ((e = cand[i].launch(fp, mode, c->d_status, c->num_sms, s))) return e;
            cudaEventRecord(c->ev1, s);
            if (cudaEventSynchronize(c->ev1) != cudaSuccess) return cudaGetLastError();
            float t = 0.f;
            cudaEventElapsedTime(&t, c->ev0, c->ev1);
            ms = t < ms ? t : ms;
        }
        if (getenv("COS_CAPON_TUNE_VERBOSE")) fprintf(stderr, "[cos_capon] tune %s: %.3f ms\n", cand[i].name, ms);
        if (ms < best_ms) {
            best_ms = ms;
            best = i;
        }
    }
    c->tuned[key] = best;
    if (getenv("COS_CAPON_TUNE_VERBOSE")) fprintf(stderr, "[cos_capon] L=%d K=%d M=%d mode=%d -> %s (%.3f ms)\n",
                                                  f0.L, f0.K, f0.M, mode, cand[best].name, best_ms);
    return cand[best].launch(fp, mode, c->d_status, c->num_sms, s);
}

// plain three-stage pipeline for one element-space frame
static int run_plain(cos_capon_ctx *c, FrameDev f, cudaStream_t s)
{
    const size_t npix = (size_t)f.Nx * f.Npy;
    int e = c->Rwork.ensure(npix * f.L * f.L * sizeof(float2));
    if (e) return e;
    if ((e = c->Ria.ensure(npix * f.L * sizeof(float2)))) return e;
    float2 *Rw = (float2 *)c->Rwork.p, *Ria = (float2 *)c->Ria.p;
    if ((e = launch_plain_build_r(f, Rw, 1, s))) return e;
    if (f.fb && (e = launch_fb_average(f, Rw, nullptr, s))) return e;
    if ((e = launch_plain_solve_hpd(f, Rw, Ria, c->d_status, s))) return e;
    if ((e = launch_plain_output(f, Ria, s))) return e;
    if (f.R) {
        // the requested R layout, written by a second covariance pass
        e = launch_plain_build_r(f, f.R, f.r_layout == COS_CAPON_R_REFERENCE ? 1 : 0, s);
        if (!e && f.fb) e = launch_fb_average(f, f.R, nullptr, s);
    }
    return e;
}

// precise pipeline (float-float covariance, FP32 Cholesky, optional FP64-residual
// refinement) for one element-space frame
static int run_precise(cos_capon_ctx *c, FrameDev f, bool refine, cudaStream_t s)
{
    const size_t npix = (size_t)f.Nx * f.Npy;
    int e;
    if ((e = c->Rwork.ensure(npix * f.L * f.L * sizeof(float2)))) return e;
    if ((e = c->Rlo.ensure(npix * f.L * f.L * sizeof(float2)))) return e;
    if ((e = c->dl.ensure(npix * sizeof(float)))) return e;
    if ((e = c->Ria.ensure(npix * f.L * sizeof(float2)))) return e;
    if ((e = launch_precise(f, (float2 *)c->Rwork.p, (float2 *)c->Rlo.p, (float *)c->dl.p, (float2 *)c->Ria.p,
                            c->d_status, refine, s)))
        return e;
    // the requested R is the float-float matrix the solve used, plus the loading
    if (f.R) e = launch_format_r(f, (float2 *)c->Rwork.p, (float2 *)c->Rlo.p, (float *)c->dl.p, f.R, s);
    return e;
}

static bool is_tc_form(int form)
{
    return form == COS_CAPON_FORM_TC_TF32 || form == COS_CAPON_FORM_TC_BF16X3 || form == COS_CAPON_FORM_TC_TF32X3;
}

// tensor-core covariance form: tcgen05 window Gram + float-float smoothing ->
// FP32 Cholesky (+ FP64-residual refinement) -> outputs
static int run_tc(cos_capon_ctx *c, FrameDev f, int split, bool refine, cudaStream_t s)
{
    const size_t npix = (size_t)f.Nx * f.Npy;
    int e;
    if ((e = c->Rwork.ensure(npix * f.L * f.L * sizeof(float2)))) return e;
    if ((e = c->dl.ensure(npix * sizeof(float)))) return e;
    if ((e = c->Ria.ensure(npix * f.L * sizeof(float2)))) return e;
    float2 *Rw = (float2 *)c->Rwork.p;
    float *dl = (float *)c->dl.p;
    if ((e = launch_tc_covariance(f, split, Rw, dl, c->d_status, c->num_sms, s))) return e;
    if (f.fb && (e = launch_fb_average(f, Rw, nullptr, s))) return e;
    if ((e = launch_precise_solve(f, Rw, nullptr, dl, (float2 *)c->Ria.p, c->d_status, refine, s))) return e;
    if (f.R) e = launch_format_r(f, Rw, nullptr, dl, f.R, s);
    return e;
}

static int run_frames(cos_capon_ctx *c, const FrameDev *fs, int n, const cos_capon_opts &o, cudaStream_t s)
{
    if (o.form < COS_CAPON_FORM_FUSED || o.form > COS_CAPON_FORM_TC_FUSED) return COS_CAPON_ERR_NOT_SUPPORTED;
    if (o.form == COS_CAPON_FORM_TC_FUSED) {
        // the tensor-core fused form: element space, z and P, shapes it is
        // instantiated for; every frame is checked before the first launch
        for (int k = 0; k < n; ++k) {
            const FrameDev &f = fs[k];
            if (f.Nb != 0 || f.fb || f.refine || f.w || f.R || !use_fused(f, o)) return COS_CAPON_ERR_NOT_SUPPORTED;
        }
    }
    if (o.form == COS_CAPON_FORM_SLIDING_INVERSE) {
        // every frame is checked before the first launch
        for (int k = 0; k < n; ++k) {
            const FrameDev &f = fs[k];
            if (f.Nb != 0 || f.fb || f.R || f.refine || f.loading != COS_CAPON_LOAD_ABSOLUTE || f.L > 32)
                return COS_CAPON_ERR_NOT_SUPPORTED;
            if (!(f.d > 0.f) || f.tile < 0) return COS_CAPON_ERR_LAUNCH;
        }
        for (int k = 0; k < n; ++k) {
            int e = launch_sliding_inverse(fs[k], c->d_status, s);
            if (e) return e;
        }
        return 0;
    }
    if (is_tc_form(o.form))
        for (int k = 0; k < n; ++k)
            if (fs[k].Nb != 0 || !tc_supported(fs[k], o.form)) return COS_CAPON_ERR_NOT_SUPPORTED;
    if (o.fb)
        for (int k = 0; k < n; ++k)
            if (fs[k].Nb > kBeamspaceTileMaxNb) return COS_CAPON_ERR_NOT_SUPPORTED;
    // Launch groups: consecutive fused frames with equal (L, K, M) share one
    // persistent launch; a beamspace frame is a group of its own; element-space
    // frames without a fused instantiation run the pipelines that use the
    // context's work buffers (R, its factor), one after another on `s`.
    struct Group {
        int kind;  // 0 fused, 1 beamspace, 2 scratch pipeline
        int first, count;
        bool want_w, want_R;
        bool scratch;  // uses context scratch (the scratch pipelines, the fused refinement modes)
        bool adaptive;  // fused: refine only the ill-conditioned pixels
        int mode() const
        {
            if (adaptive) return want_w ? FUSED_ADAPT_W : FUSED_ADAPT_ZP;
            return scratch ? FUSED_REFINE : want_w ? FUSED_W : FUSED_ZP;
        }
    };
    std::vector<Group> groups;
    for (int i = 0; i < n;) {
        const FrameDev &f = fs[i];
        if (use_fused(f, o)) {
            Group g{0, i, 0, false, false, o.refine != 0, o.refine == COS_CAPON_REFINE_ADAPTIVE};
            int j = i;
            while (j < n && g.count < kMaxFrames && use_fused(fs[j], o) && fs[j].L == f.L && fs[j].K == f.K &&
                   fs[j].M == f.M) {
                g.want_w |= fs[j].w != nullptr;
                g.want_R |= fs[j].R != nullptr;
                ++g.count;
                ++j;
            }
            groups.push_back(g);
            i = j;
        } else {
            groups.push_back(Group{f.Nb > 0 ? 1 : 2, i, 1, false, false, f.Nb == 0, false});
            ++i;
        }
    }
    auto launch_group = [&](const Group &g, cudaStream_t st) -> int {
        const FrameDev &f = fs[g.first];
        if (g.kind == 0) {
            FramesParam fp;
            memset(&fp, 0, sizeof(fp));
            const char *stall = getenv("COS_CAPON_TEST_STALL");
            fp.stall_test = stall && stall[0] == '1';
            for (int q = 0; q < g.count; ++q) fp.f[fp.n++] = fs[g.first + q];
            // R, when asked for, comes from its own covariance pass; z, P (and w)
            // from the factorising launch
            if (g.want_R) {
                if (int e = launch_fused_tuned(c, fp, FUSED_R, o.form, st)) return e;
            }
            if (g.scratch) {
                // the stash for the largest candidate of the shape
                const FusedCandidate *cand = nullptr;
                const int nc = candidates(f.L, f.K, o.form, &cand);
                size_t need = 0;
                for (int q = 0; q < nc; ++q)
                    if (cand_fits(cand[q], f, true)) need = std::max(need, cand[q].stash(c->num_sms));
                if (need == 0) return COS_CAPON_ERR_NOT_SUPPORTED;
                if (int e = c->stash.ensure(need)) return e;
                fp.stash = (float4 *)c->stash.p;
                fp.stash_bytes = c->stash.cap;
            }
            return launch_fused_tuned(c, fp, g.mode(), o.form, st);
        }
        if (g.kind == 1) {
            int e = launch_beamspace(f, nullptr, st);
            if (e) return e;
            if (f.R) {  // element-space loaded R, as the reference copies it back (Capon.cpp:253-259)
                FrameDev h = f;
                h.Nb = 0;
                e = launch_plain_build_r(h, f.R, f.r_layout == COS_CAPON_R_REFERENCE ? 1 : 0, st);
            }
            return e;
        }
        // element space without a fused instantiation (or with refinement):
        // the precise pipeline; the plain form when asked for
        return is_tc_form(o.form)                              ? run_tc(c, f, o.form, o.refine != 0, st)
               : (o.form == COS_CAPON_FORM_PLAIN && !o.refine) ? run_plain(c, f, st)
                                                               : run_precise(c, f, o.refine != 0, st);
    };
    // Groups that use no context scratch (fused, beamspace) may run side by
    // side: the first on `s`, the next ones on the auxiliary streams, forked
    // from `s` and joined back by events, so that one kernel's tail overlaps
    // the next one's start (captured, they become parallel graph branches).
    // Not while an untuned fused shape is timed by the autotuner.
    std::vector<int> free_groups, scratch_groups;
    bool tuned_all = true;
    for (int k = 0; k < (int)groups.size(); ++k) {
        const Group &g = groups[k];
        (g.scratch ? scratch_groups : free_groups).push_back(k);
        if (g.kind == 0) {
            const FrameDev &f = fs[g.first];
            const int mode = g.mode();
            tuned_all &= c->tuned.count(std::make_tuple(f.L, f.K, f.M, mode | (o.form << 8))) != 0;
            if (g.want_R) tuned_all &= c->tuned.count(std::make_tuple(f.L, f.K, f.M, FUSED_R | (o.form << 8))) != 0;
        }
    }
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    if (cudaStreamIsCapturing(s, &cs) != cudaSuccess) {
        cudaGetLastError();
        cs = cudaStreamCaptureStatusNone;
    }
    const bool side_by_side = free_groups.size() > 1 && c->fork_ev &&
                              (tuned_all || cs != cudaStreamCaptureStatusNone) &&
                              !getenv("COS_CAPON_SERIAL_FRAMES");
    if (!side_by_side) {
        for (const Group &g : groups)
            if (int e = launch_group(g, s)) return e;
        return 0;
    }
    const int naux = std::min((int)free_groups.size() - 1, cos_capon_ctx::kAux);
    cudaError_t ce = cudaEventRecord(c->fork_ev, s);
    for (int k = 0; k < naux && ce == cudaSuccess; ++k) ce = cudaStreamWaitEvent(c->aux[k], c->fork_ev, 0);
    if (ce != cudaSuccess) return ce;
    int err = 0;
    for (int q = 0; q < (int)free_groups.size() && !err; ++q) {
        // group 0 and the ones past the auxiliary streams on `s`
        const cudaStream_t st = (q >= 1 && q <= naux) ? c->aux[q - 1] : s;
        err = launch_group(groups[free_groups[q]], st);
    }
    // join every auxiliary stream back into `s`, also after an error
    for (int k = 0; k < naux; ++k) {
        cudaError_t je = cudaEventRecord(c->join_ev[k], c->aux[k]);
        if (je == cudaSuccess) je = cudaStreamWaitEvent(s, c->join_ev[k], 0);
        if (je != cudaSuccess && !err) err = je;
    }
    if (err) return err;
    for (int k : scratch_groups)
        if (int e = launch_group(groups[k], s)) return e;
    return 0;
}

static bool is_pinned(const void *p)
{
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    return a.type == cudaMemoryTypeHost;
}

static int read_status(cos_capon_ctx *c, cudaStream_t s, bool sync)
{
    if (sync) {
        cudaError_t e = cudaStreamSynchronize(s);
        if (e != cudaSuccess) return e;
    }
    unsigned st = 0;
    cudaError_t e = cudaMemcpy(&st, c->d_status, sizeof(unsigned), cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) return e;
    if (st & ERR_TIMEOUT) {
        cudaMemset(c->d_status, 0, sizeof(unsigned));
        return COS_CAPON_ERR_TIMEOUT;
    }
    return 0;
}

extern "C" {

int cos_capon_create(cos_capon_ctx **ctx)
{
    if (!ctx) return COS_CAPON_ERR_INVALID_VALUE;
    *ctx = nullptr;
    cos_capon_ctx *c = new (std::nothrow) cos_capon_ctx();
    if (!c) return COS_CAPON_ERR_OUT_OF_MEMORY;
    cudaError_t e = cudaGetDevice(&c->device);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&c->num_sms, cudaDevAttrMultiProcessorCount, c->device);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaMalloc(&c->d_status, sizeof(unsigned));
    if (e == cudaSuccess) e = cudaMemset(c->d_status, 0, sizeof(unsigned));
    for (int k = 0; k < cos_capon_ctx::kAux && e == cudaSuccess; ++k) {
        e = cudaStreamCreateWithFlags(&c->aux[k], cudaStreamNonBlocking);
        if (e == cudaSuccess) e = cudaEventCreateWithFlags(&c->join_ev[k], cudaEventDisableTiming);
    }
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&c->fork_ev, cudaEventDisableTiming);
    if (e != cudaSuccess) {
        cudaGetLastError();
        if (c->stream) cudaStreamDestroy(c->stream);
        if (c->d_status) cudaFree(c->d_status);
        for (int k = 0; k < cos_capon_ctx::kAux; ++k) {
            if (c->aux[k]) cudaStreamDestroy(c->aux[k]);
            if (c->join_ev[k]) cudaEventDestroy(c->join_ev[k]);
        }
        if (c->fork_ev) cudaEventDestroy(c->fork_ev);
        delete c;
        return e;
    }
    *ctx = c;
    return 0;
}

int cos_capon_destroy(cos_capon_ctx *c)
{
    if (!c) return COS_CAPON_ERR_INVALID_VALUE;
    cudaStreamSynchronize(c->stream);
    for (DevBuf *b : {&c->x, &c->z, &c->P, &c->w, &c->R, &c->Rwork, &c->Rlo, &c->dl, &c->Ria, &c->stash, &c->A,
                      &c->b, &c->sol, &c->V, &c->tdib_in, &c->lca_pw})
        b->release();
    if (c->d_status) cudaFree(c->d_status);
    if (c->stream) cudaStreamDestroy(c->stream);
    if (c->stream2) cudaStreamDestroy(c->stream2);
    if (c->ev0) cudaEventDestroy(c->ev0);
    if (c->ev1) cudaEventDestroy(c->ev1);
    for (int k = 0; k < cos_capon_ctx::kAux; ++k) {
        if (c->aux[k]) cudaStreamDestroy(c->aux[k]);
        if (c->join_ev[k]) cudaEventDestroy(c->join_ev[k]);
    }
    if (c->fork_ev) cudaEventDestroy(c->fork_ev);
    delete c;
    return 0;
}

int cos_capon_run(cos_capon_ctx *c, const cos_capon_frame *frames, int nframes, const cos_capon_opts *opts,
                  void *stream)
{
    if (!c || !frames || nframes < 1) return COS_CAPON_ERR_INVALID_VALUE;
    const cos_capon_opts o = opts ? *opts : kDefaultOpts;
    std::vector<FrameDev> fs;
    fs.reserve(nframes);
    for (int i = 0; i < nframes; ++i) {
        const cos_capon_frame &fr = frames[i];
        int e = check_sizes(fr.L, fr.K, fr.M, fr.Nx, fr.Ny, fr.Nb);
        if (e) return e;
        if (!fr.x || !fr.z) return COS_CAPON_ERR_INVALID_VALUE;
        fs.push_back(make_frame(fr, o));
    }
    // NULL is the default stream, as everywhere in CUDA; the context's own
    // stream serves only the host-pointer calls
    cudaStream_t s = (cudaStream_t)stream;
    return run_frames(c, fs.data(), nframes, o, s);
}

// the host-pointer call; V (host, [Nb][L]) selects a caller-given subspace
static int get_capon_host(cos_capon_ctx *c, void *z, float *P, void *w, void *R, const void *x, const void *V,
                          float d, int L, int Yavg, int M, int Nx, int Nz, int Nb, const cos_capon_opts *opts)
{
    if (!c) return COS_CAPON_ERR_INVALID_VALUE;
    int e = check_sizes(L, Yavg, M, Nx, Nz, Nb);
    if (e) return e;
    if (!x || !z) return COS_CAPON_ERR_INVALID_VALUE;
    if (V && Nb < 1) return COS_CAPON_ERR_INVALID_VALUE;
    const cos_capon_opts o = opts ? *opts : kDefaultOpts;
    const size_t N = (size_t)Nx * Nz, npix = (size_t)Nx * (Nz - 2 * Yavg);
    const size_t bx = N * M * sizeof(float2), bz = npix * sizeof(float2), bp = npix * sizeof(float),
                 bw = npix * L * sizeof(float2), bR = npix * L * L * sizeof(float2);
    cos_capon_frame probe;
    memset(&probe, 0, sizeof(probe));
    probe.L = L;
    probe.K = Yavg;
    probe.M = M;
    probe.Nb = Nb;
    const bool plain = !use_fused(make_frame(probe, o), o);
    size_t need = 0;
    need += bx > c->x.cap ? bx : 0;
    need += bz > c->z.cap ? bz : 0;
    need += (P && bp > c->P.cap) ? bp : 0;
    need += (w && bw > c->w.cap) ? bw : 0;
    need += (R && bR > c->R.cap) ? bR : 0;
    const bool sliding = o.form == COS_CAPON_FORM_SLIDING_INVERSE;
    if (plain && Nb == 0 && !sliding) {
        need += (bR > c->Rwork.cap ? bR : 0) + (bw > c->Ria.cap ? bw : 0);
        if (!(o.form == COS_CAPON_FORM_PLAIN && !o.refine)) need += bR > c->Rlo.cap ? bR : 0;
    }
    if ((e = check_free(need))) return e;
    if ((e = c->x.ensure(bx)) || (e = c->z.ensure(bz))) return e;
    if (P && (e = c->P.ensure(bp))) return e;
    if (w && (e = c->w.ensure(bw))) return e;
    if (R && (e = c->R.ensure(bR))) return e;

    cudaStream_t s = c->stream;
    cudaError_t ce;
    const void *Vd = nullptr;
    if (V) {
        const size_t bv = (size_t)Nb * L * sizeof(float2);
        if ((e = c->V.ensure(bv))) return e;
        if ((ce = cudaMemcpyAsync(c->V.p, V, bv, cudaMemcpyHostToDevice, s)) != cudaSuccess) return ce;
        Vd = c->V.p;
    }
    // Pinned host buffers and a path without shared scratch (fused, beamspace):
    // split the beams into chunks on two streams so that the copies of one
    // chunk overlap the kernel of the other.  The first call of a fused shape
    // runs whole, so the autotuner times the frame once, on one stream.
    const bool fused = use_fused(make_frame(probe, o), o);
    const bool no_scratch = (fused && !o.refine) || Nb > 0 || sliding;
    const bool tuned = !fused || c->tuned.count(std::make_tuple(L, Yavg, M, (int)(w ? FUSED_W : FUSED_ZP) | (o.form << 8)));
    if (no_scratch && tuned && !R && !V && Nx >= 4 && is_pinned(x) && is_pinned(z) && (!P || is_pinned(P)) &&
        (!w || is_pinned(w))) {
        if (!c->stream2 && cudaStreamCreateWithFlags(&c->stream2, cudaStreamNonBlocking) != cudaSuccess) {
            cudaGetLastError();
            c->stream2 = nullptr;
        }
        if (c->stream2) {
            const int nch = Nx >= 16 ? 8 : Nx / 2;
            const size_t rowx = (size_t)Nz * M, rowp = (size_t)(Nz - 2 * Yavg);
            for (int ch = 0; ch < nch; ++ch) {
                const int b0 = (int)((long)Nx * ch / nch), b1 = (int)((long)Nx * (ch + 1) / nch);
                cudaStream_t sc = (ch & 1) ? c->stream2 : c->stream;
                const size_t nb = (size_t)(b1 - b0);
                if ((ce = cudaMemcpyAsync((float2 *)c->x.p + b0 * rowx, (const float2 *)x + b0 * rowx,
                                          nb * rowx * sizeof(float2), cudaMemcpyHostToDevice, sc)) != cudaSuccess)
                    return ce;
                cos_capon_frame fr;
                memset(&fr, 0, sizeof(fr));
                fr.x = (float2 *)c->x.p + b0 * rowx;
                fr.z = (float2 *)c->z.p + b0 * rowp;
                fr.P = P ? (float *)c->P.p + b0 * rowp : nullptr;
                fr.w = w ? (float2 *)c->w.p + b0 * rowp * L : nullptr;
                fr.d = d;
                fr.L = L;
                fr.K = Yavg;
                fr.M = M;
                fr.Nx = (int)nb;
                fr.Ny = Nz;
                fr.Nb = Nb;
                if ((e = cos_capon_run(c, &fr, 1, &o, sc))) return e;
                if ((ce = cudaMemcpyAsync((float2 *)z + b0 * rowp, fr.z, nb * rowp * sizeof(float2),
                                          cudaMemcpyDeviceToHost, sc)) != cudaSuccess)
                    return ce;
                if (P && (ce = cudaMemcpyAsync(P + b0 * rowp, fr.P, nb * rowp * sizeof(float), cudaMemcpyDeviceToHost,
                                               sc)) != cudaSuccess)
                    return ce;
                if (w && (ce = cudaMemcpyAsync((float2 *)w + b0 * rowp * L, fr.w, nb * rowp * L * sizeof(float2),
                                               cudaMemcpyDeviceToHost, sc)) != cudaSuccess)
                    return ce;
            }
            if ((ce = cudaStreamSynchronize(c->stream2)) != cudaSuccess) return ce;
            return read_status(c, s, true);
        }
    }
    if ((ce = cudaMemcpyAsync(c->x.p, x, bx, cudaMemcpyHostToDevice, s)) != cudaSuccess) return ce;
    cos_capon_frame fr;
    memset(&fr, 0, sizeof(fr));
    fr.V = Vd;
    fr.x = c->x.p;
    fr.z = c->z.p;
    fr.P = P ? (float *)c->P.p : nullptr;
    fr.w = w ? c->w.p : nullptr;
    fr.R = R ? c->R.p : nullptr;
    fr.d = d;
    fr.L = L;
    fr.K = Yavg;
    fr.M = M;
    fr.Nx = Nx;
    fr.Ny = Nz;
    fr.Nb = Nb;
    if ((e = cos_capon_run(c, &fr, 1, &o, s))) return e;
    if ((ce = cudaMemcpyAsync(z, c->z.p, bz, cudaMemcpyDeviceToHost, s)) != cudaSuccess) return ce;
    if (P && (ce = cudaMemcpyAsync(P, c->P.p, bp, cudaMemcpyDeviceToHost, s)) != cudaSuccess) return ce;
    if (w && (ce = cudaMemcpyAsync(w, c->w.p, bw, cudaMemcpyDeviceToHost, s)) != cudaSuccess) return ce;
    if (R && (ce = cudaMemcpyAsync(R, c->R.p, bR, cudaMemcpyDeviceToHost, s)) != cudaSuccess) return ce;
    return read_status(c, s, true);
}

int cos_capon_get_capon_ex(cos_capon_ctx *c, void *z, float *P, void *w, void *R, const void *x, float d, int L,
                           int Yavg, int M, int Nx, int Nz, int Nb, const cos_capon_opts *opts)
{
    return get_capon_host(c, z, P, w, R, x, nullptr, d, L, Yavg, M, Nx, Nz, Nb, opts);
}

int cos_capon_get_capon_subspace(cos_capon_ctx *c, void *z, float *P, void *w, const void *x, const void *V, float d,
                                 int L, int Yavg, int M, int Nx, int Nz, int Nb, const cos_capon_opts *opts)
{
    if (!V) return COS_CAPON_ERR_INVALID_VALUE;
    return get_capon_host(c, z, P, w, nullptr, x, V, d, L, Yavg, M, Nx, Nz, Nb, opts);
}

int cos_capon_tdib(cos_capon_ctx *c, const void *mfdata, int n_hydros, int n_samples, double t0, double dt,
                   const double *x_r, const double *D, double cs, double fc, const double *xarr, const double *yarr,
                   int n_x, int n_y, void *Xd, void *image, int on_gpu, void *stream)
{
    if (!c || !mfdata || !x_r || !D || !xarr || !yarr || (!Xd && !image)) return COS_CAPON_ERR_INVALID_VALUE;
    if (n_hydros < 1 || n_samples < 2 || n_x < 1 || n_y < 1 || !(dt > 0.0) || !(cs > 0.0))
        return COS_CAPON_ERR_LAUNCH;
    TdibDev t;
    memset(&t, 0, sizeof(t));
    t.t0 = t0;
    t.dt = dt;
    t.inv_c = 1.0 / cs;
    t.fc = fc;
    t.n_hydros = n_hydros;
    t.n_samples = n_samples;
    t.n_x = n_x;
    t.n_y = n_y;
    const size_t bmf = (size_t)n_hydros * n_samples * sizeof(float2), bh = (size_t)n_hydros * sizeof(double),
                 bg = (size_t)n_x * n_y * sizeof(double), bXd = (size_t)n_x * n_y * n_hydros * sizeof(float2),
                 bimg = (size_t)n_x * n_y * sizeof(float2);
    if (on_gpu) {
        t.mf = (const float2 *)mfdata;
        t.x_r = x_r;
        t.D = D;
        t.xarr = xarr;
        t.yarr = yarr;
        t.Xd = (float2 *)Xd;
        t.image = (float2 *)image;
        return launch_tdib(t, (cudaStream_t)stream);
    }
    // host pointers: inputs through the context's buffers, synchronous
    int e;
    const size_t bin = bmf + 2 * bh + 2 * bg;
    if ((e = check_free((bin > c->tdib_in.cap ? bin : 0) + (Xd && bXd > c->x.cap ? bXd : 0) +
                        (image && bimg > c->z.cap ? bimg : 0))))
        return e;
    if ((e = c->tdib_in.ensure(bin))) return e;
    if (Xd && (e = c->x.ensure(bXd))) return e;
    if (image && (e = c->z.ensure(bimg))) return e;
    cudaStream_t s = c->stream;
    unsigned char *in = (unsigned char *)c->tdib_in.p;
    cudaError_t ce;
    const void *src[5] = {x_r, D, xarr, yarr, mfdata};
    const size_t len[5] = {bh, bh, bg, bg, bmf};
    size_t off = 0;
    for (int k = 0; k < 5; ++k) {
        if ((ce = cudaMemcpyAsync(in + off, src[k], len[k], cudaMemcpyHostToDevice, s)) != cudaSuccess) return ce;
        off += len[k];
    }
    t.x_r = (const double *)in;
    t.D = (const double *)(in + bh);
    t.xarr = (const double *)(in + 2 * bh);
    t.yarr = (const double *)(in + 2 * bh + bg);
    t.mf = (const float2 *)(in + 2 * bh + 2 * bg);
    t.Xd = Xd ? (float2 *)c->x.p : nullptr;
    t.image = image ? (float2 *)c->z.p : nullptr;
    if ((e = launch_tdib(t, s))) return e;
    if (Xd && (ce = cudaMemcpyAsync(Xd, c->x.p, bXd, cudaMemcpyDeviceToHost, s)) != cudaSuccess) return ce;
    if (image && (ce = cudaMemcpyAsync(image, c->z.p, bimg, cudaMemcpyDeviceToHost, s)) != cudaSuccess) return ce;
    return read_status(c, s, true);
}

int cos_capon_lca(cos_capon_ctx *c, const void *Z, int Ny, int Nx, int Nw, const double *wrf, int Yf, int Xf,
                  void *img, int *win, int on_gpu, void *stream)
{
    if (!c || !Z || !wrf || !img) return COS_CAPON_ERR_INVALID_VALUE;
    if (Ny < 1 || Nx < 1 || Nw < 1 || Yf < 1 || Xf < 1 || !(Yf & 1) || !(Xf & 1) || Yf * Xf > kLcaMaxFilter)
        return COS_CAPON_ERR_LAUNCH;
    LcaDev a;
    memset(&a, 0, sizeof(a));
    a.Ny = Ny;
    a.Nx = Nx;
    a.Nw = Nw;
    a.Yf = Yf;
    a.Xf = Xf;
    a.Ymid = (Yf - 1) / 2;
    a.Xmid = (Xf - 1) / 2;
    a.single = (Yf == 1 && Xf == 1 && wrf[0] != 0.0);
    for (int i = 0; i < Yf * Xf; ++i) a.wrf[i] = (float)wrf[i];
    const size_t bZ = (size_t)Ny * Nx * Nw * sizeof(float2), bpw = (size_t)Ny * Nx * Nw * sizeof(float),
                 bimg = (size_t)Ny * Nx * sizeof(float2), bwin = (size_t)Ny * Nx * sizeof(int);
    int e;
    if ((e = check_free((bpw > c->lca_pw.cap ? bpw : 0) +
                        (on_gpu ? 0 : (bZ > c->x.cap ? bZ : 0) + (bimg > c->z.cap ? bimg : 0) +
                                          (win && bwin > c->P.cap ? bwin : 0)))))
        return e;
    if ((e = c->lca_pw.ensure(bpw))) return e;   // |Z|^2 planes
    if (on_gpu) {
        a.Z = (const float2 *)Z;
        a.img = (float2 *)img;
        a.win = win;
        return launch_lca(a, (float *)c->lca_pw.p, (cudaStream_t)stream);
    }
    if ((e = c->x.ensure(bZ)) || (e = c->z.ensure(bimg))) return e;
    if (win && (e = c->P.ensure(bwin))) return e;
    cudaStream_t s = c->stream;
    cudaError_t ce;
    if ((ce = cudaMemcpyAsync(c->x.p, Z, bZ, cudaMemcpyHostToDevice, s)) != cudaSuccess) return ce;
    a.Z = (const float2 *)c->x.p;
    a.img = (float2 *)c->z.p;
    a.win = win ? (int *)c->P.p : nullptr;
    if ((e = launch_lca(a, (float *)c->lca_pw.p, s))) return e;
    if ((ce = cudaMemcpyAsync(img, c->z.p, bimg, cudaMemcpyDeviceToHost, s)) != cudaSuccess) return ce;
    if (win && (ce = cudaMemcpyAsync(win, c->P.p, bwin, cudaMemcpyDeviceToHost, s)) != cudaSuccess) return ce;
    return read_status(c, s, true);
}

int cos_capon_get_capon(cos_capon_ctx *c, void *z, void *w, void *R, const void *x, float d, int L, int Yavg, int M,
                        int Nx, int Nz, int Nb)
{
    if (!w) return COS_CAPON_ERR_INVALID_VALUE;
    return cos_capon_get_capon_ex(c, z, nullptr, w, R, x, d, L, Yavg, M, Nx, Nz, Nb, nullptr);
}

int cos_capon_build_r(cos_capon_ctx *c, void *R, const void *x, float d, int L, int Yavg, int M, int Nx, int Nz,
                      int Nb, int R_on_gpu, int x_on_gpu)
{
    if (!c || !R || !x) return COS_CAPON_ERR_INVALID_VALUE;
    int e = check_sizes(L, Yavg, M, Nx, Nz, Nb);
    if (e) return e;
    const int n = Nb > 0 ? Nb : L;
    const size_t npix = (size_t)Nx * (Nz - 2 * Yavg);
    const size_t bx = (size_t)Nx * Nz * M * sizeof(float2), bR = npix * n * n * sizeof(float2);
    cudaStream_t s = c->stream;
    const void *xd = x;
    void *Rd = R;
    cudaError_t ce;
    if (!x_on_gpu) {
        if ((e = c->x.ensure(bx))) return e;
        if ((ce = cudaMemcpyAsync(c->x.p, x, bx, cudaMemcpyHostToDevice, s)) != cudaSuccess) return ce;
        xd = c->x.p;
    }
    if (!R_on_gpu) {
        if ((e = c->R.ensure(bR))) return e;
        Rd = c->R.p;
    }
    cos_capon_frame fr;
    memset(&fr, 0, sizeof(fr));
    fr.x = xd;
    fr.d = d;
    fr.L = L;
    fr.K = Yavg;
    fr.M = M;
    fr.Nx = Nx;
    fr.Ny = Nz;
    fr.Nb = Nb;
    cos_capon_opts o = kDefaultOpts;
    FrameDev f = make_frame(fr, o);
    if (Nb > 0) {
        // the reference's beamspace BuildR loads with tr(R_bs)/Nb (BuildR.cpp:82-86)
        f.loading = COS_CAPON_LOAD_BEAMSPACE;
        if ((e = launch_beamspace(f, (float2 *)Rd, s))) return e;
    } else {
        if ((e = launch_plain_build_r(f, (float2 *)Rd, 1, s))) return e;
    }
    if (!R_on_gpu && (ce = cudaMemcpyAsync(R, Rd, bR, cudaMemcpyDeviceToHost, s)) != cudaSuccess) return ce;
    return read_status(c, s, true);
}

int cos_capon_solve(cos_capon_ctx *c, void *x, const void *A, const void *b, int N, int batch, int x_on_gpu,
                    int A_on_gpu, int b_on_gpu)
{
    if (!c || !x || !A || !b) return COS_CAPON_ERR_INVALID_VALUE;
    // Solver.cpp:34-42
    if (N < 1 || N > 72 || batch < 1) return COS_CAPON_ERR_LAUNCH;
    const size_t bA = (size_t)N * N * batch * sizeof(float2), bv = (size_t)N * batch * sizeof(float2);
    cudaStream_t s = c->stream;
    cudaError_t ce;
    int e;
    const void *Ad = A, *bd = b;
    void *xd = x;
    if (!A_on_gpu) {
        if ((e = c->A.ensure(bA))) return e;
        if ((ce = cudaMemcpyAsync(c->A.p, A, bA, cudaMemcpyHostToDevice, s)) != cudaSuccess) return ce;
        Ad = c->A.p;
    }
    if (!b_on_gpu) {
        if ((e = c->b.ensure(bv))) return e;
        if ((ce = cudaMemcpyAsync(c->b.p, b, bv, cudaMemcpyHostToDevice, s)) != cudaSuccess) return ce;
        bd = c->b.p;
    }
    if (!x_on_gpu) {
        if ((e = c->sol.ensure(bv))) return e;
        xd = c->sol.p;
    }
    if ((e = launch_lu_solve((float2 *)xd, (const float2 *)Ad, (const float2 *)bd, N, batch, s))) return e;
    if (!x_on_gpu && (ce = cudaMemcpyAsync(x, xd, bv, cudaMemcpyDeviceToHost, s)) != cudaSuccess) return ce;
    return read_status(c, s, true);
}

int cos_capon_butler(cos_capon_ctx *c, void *B, int Nb, int L, int B_on_gpu)
{
    if (!c || !B) return COS_CAPON_ERR_INVALID_VALUE;
    if (Nb < 1 || L < 1 || Nb > L) return COS_CAPON_ERR_LAUNCH;
    const size_t bytes = (size_t)Nb * L * sizeof(float2);
    cudaStream_t s = c->stream;
    void *Bd = B;
    int e;
    if (!B_on_gpu) {
        if ((e = c->sol.ensure(bytes))) return e;
        Bd = c->sol.p;
    }
    if ((e = launch_butler((float2 *)Bd, Nb, L, s))) return e;
    cudaError_t ce;
    if (!B_on_gpu && (ce = cudaMemcpyAsync(B, Bd, bytes, cudaMemcpyDeviceToHost, s)) != cudaSuccess) return ce;
    return read_status(c, s, true);
}

int cos_capon_backward(cos_capon_ctx *c, const cos_capon_adjoint *adj, void *stream)
{
    if (!c || !adj || !adj->x || !adj->w || !adj->gP || !adj->gx) return COS_CAPON_ERR_INVALID_VALUE;
    int e = check_sizes(adj->L, adj->K, adj->M, adj->Nx, adj->Ny, 0);
    if (e) return e;
    AdjDev a;
    a.x = (const float2 *)adj->x;
    a.w = (const float2 *)adj->w;
    a.gP = adj->gP;
    a.gx = (float2 *)adj->gx;
    a.gd = adj->gd;
    a.gth = adj->gtheta;
    a.L = adj->L;
    a.K = adj->K;
    a.M = adj->M;
    a.Nx = adj->Nx;
    a.Ny = adj->Ny;
    a.Npy = adj->Ny - 2 * adj->K;
    return launch_adjoint(a, c->num_sms, (cudaStream_t)stream);
}

int cos_capon_device_status(cos_capon_ctx *c)
{
    if (!c) return COS_CAPON_ERR_INVALID_VALUE;
    return read_status(c, c->stream, true);
}

const char *cos_capon_status_string(int st)
{
    switch (st) {
    case COS_CAPON_SUCCESS: return "success";
    case COS_CAPON_ERR_INVALID_VALUE: return "invalid value (NULL context or buffer)";
    case COS_CAPON_ERR_OUT_OF_MEMORY: return "not enough device memory for the requested sizes";
    case COS_CAPON_ERR_LAUNCH: return "invalid sizes (Nx, Nz, L, M < 1; Yavg, Nb < 0; Nb > L; L > M; 2*Yavg >= Nz; N outside [1, 72])";
    case COS_CAPON_ERR_NOT_SUPPORTED: return "option or size outside what this build implements";
    case COS_CAPON_ERR_TIMEOUT: return "a bounded device-side wait expired";
    default: return cudaGetErrorString((cudaError_t)st);
    }
}

}  // extern "C"
