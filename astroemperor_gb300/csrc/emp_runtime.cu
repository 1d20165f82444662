// emp_runtime.cu -- host runtime behind the C ABI of include/emp_gpu.h.
//
// Owns: descriptor validation, the device dataset layout, launch-shape
// selection, kernel dispatch, the PT sweep sequence and its CUDA-graph
// cache.  No exception crosses the ABI; every entry returns a status.
#include <cuda_runtime.h>
#include <math.h>
#include <stdio.h>
#include <string.h>

#include <algorithm>
#include <atomic>
#include <cstdarg>
#include <mutex>
#include <numeric>
#include <vector>

#include "emp_device.cuh"
#include "emp_pt.cuh"
#include "emp_model_eval.cuh"
#include "emp_grad.cuh"
#include "emp_gp.cuh"

namespace emp {
using KFn = void (*)(KArgs);
KFn get_kernel_fp64(int q, int lidx);
KFn get_kernel_mixed(int q, int lidx);
using GFn = void (*)(GArgs);
GFn get_kernel_grad(int q, int lidx);
KFn get_kernel_gp(int M, int prep, int ff);
KFn get_kernel_am(int prec);
}  // namespace emp

using namespace emp;

namespace {

thread_local char g_err[512] = "";
std::atomic<int64_t> g_launches{0};

int fail(int code, const char* fmt, ...) {
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(g_err, sizeof(g_err), fmt, ap);
    va_end(ap);
    return code;
}

#define CUDA_TRY(expr)                                                          \
    do {                                                                        \
        cudaError_t _e = (expr);                                                \
        if (_e != cudaSuccess)                                                  \
            return fail(EMP_E_CUDA, "%s failed: %s", #expr, cudaGetErrorString(_e)); \
    } while (0)

const int kLanes[6] = {8, 16, 32, 64, 128, 256};

int lanes_index(int L) {
    for (int i = 0; i < 6; ++i)
        if (kLanes[i] == L) return i;
    return -1;
}

struct GraphCache {
    bool valid = false;
    emp_pt_state st{};
    emp_pt_record rec{};
    bool has_rec = false;
    cudaStream_t stream = nullptr;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    void* host = nullptr;        // packed host state copied in and out (emp_pt_run_host)
    int kernels_per_launch = 0;
    void reset() {
        if (exec) cudaGraphExecDestroy(exec);
        if (graph) cudaGraphDestroy(graph);
        exec = nullptr;
        graph = nullptr;
        valid = false;
    }
};

}  // namespace

struct emp_handle {
    emp_model_desc md{};       // system 0 (the only one unless batched)
    emp_model_desc* md_dev = nullptr;   // [n_sys]
    int n = 0;                 // epochs of the largest system (tile size)
    int n_typ = 0;             // median epochs per system (default lanes)
    int n_sys = 1;
    int lay[5] = {};           // largest n_full, n_free, n_planets, n_ins, acc_order
    const int64_t* sys_off = nullptr;   // device [S+1] epoch offsets (batch only)
    const double* sys_t0 = nullptr;     // device [S] acceleration origins (batch only)
    const int* sys_order = nullptr;     // device [S] costliest system first (batch only)
    int persist_grid[2][6] = {};
    int persist_smem[2][6] = {};
    int q = 0;                 // MA order evaluated on device
    void* dbuf = nullptr;
    DevData dd{};
    int L[2] = {0, 0};
    int tile[2] = {0, 0};
    int* dev2orig = nullptr;
    cudaStream_t own = nullptr;
    GraphCache gc;               // emp_pt_run
    GraphCache gch;              // emp_pt_run_host
    cudaStream_t aux = nullptr;  // second stream of the host-state graph
    bool attr_done[2][4][6] = {};
    bool swap_attr = false;
    bool swap_attr_batch = false;
    // celerite GP likelihood: state dimension of k_gp (0: Gaussian likelihood)
    // and its row buffers (residuals and err2 [n][rows], proposals, meta)
    int gp_M = 0;
    int64_t gp_rows = 0;
    void* gp_buf = nullptr;
    double* gp_r = nullptr;
    double* gp_e = nullptr;
    double* gp_prop = nullptr;
    GPMeta* gp_meta = nullptr;
    double* gp_u = nullptr;
    double* gp_v = nullptr;
    double* gp_ph = nullptr;
    double* gp_asum = nullptr;
    int sms = 0;
    // adjoint kernel: epoch tile (0: chosen per call) and the residual buffer
    // of MA models whose series spans several tiles (grown on demand)
    int grad_tile = 0;
    bool grad_attr[4] = {};      // the adjoint kernel's shared-memory limit set, by MA order
    void* grad_buf = nullptr;
    size_t grad_bytes = 0;
    // joint astrometry (md.am_on): the data on the device, and per walker
    // row of a stretch half-step the proposal, its meta and its RV logL
    bool am_set = false;
    AmDev am{};
    const AmDev* am_sys = nullptr;   // [S] on the device, a batch handle's per-system data
    void* am_buf = nullptr;
    void* am_rows_buf = nullptr;
    int64_t am_rows = 0;
    double* am_rv = nullptr;
    double* am_prop = nullptr;
    GPMeta* am_meta = nullptr;
};

// dynamic shared memory of the staged swap kernel (static arrays use ~12 KB)
static const size_t kSwapSmemMax = 200 * 1024;
// history rows of one sweep up to this size are written by the swap CTA (one
// SM writes ~20 GB/s: measured 39.6 -> 35.5 us per sweep for 2 x 100 walkers
// (14 KB of rows), but 82 -> 107 us for 10 x 256 (512 KB))
static const size_t kRecInSwapMax = 64 * 1024;
// threads per CTA of the GP recursion (M lanes per walker row): one warp,
// so that the recursion's warps spread over the SMs (measured 5 % faster
// than four warps per CTA for 1280 rows; FP64 issue is per SM sub-partition)
static const int kGPBlock = 32;

namespace {

int validate_prior(const emp_prior& p, const char* what, int i) {
    if (p.kind < EMP_PRIOR_UNIFORM || p.kind > EMP_PRIOR_ISOTROPIC)
        return fail(EMP_E_INVALID, "%s %d: unknown prior kind %d", what, i, p.kind);
    if (p.kind == EMP_PRIOR_NONE) return EMP_OK;
    if (!(p.lo <= p.hi)) return fail(EMP_E_INVALID, "%s %d: limits not ordered", what, i);
    if (p.kind == EMP_PRIOR_NORMAL && !(p.a1 > 0))
        return fail(EMP_E_INVALID, "%s %d: Normal 1/scale must be > 0", what, i);
    return EMP_OK;
}

int validate_model(const emp_model_desc* m) {
    if (!m) return fail(EMP_E_INVALID, "model descriptor is NULL");
    if (m->abi_version != EMP_ABI_VERSION)
        return fail(EMP_E_INVALID, "descriptor ABI %d, library ABI %d", m->abi_version, EMP_ABI_VERSION);
    if (m->n_full < 0 || m->n_full > EMP_MAX_PARAMS)
        return fail(EMP_E_SIZE, "n_full=%d outside [0, %d]", m->n_full, EMP_MAX_PARAMS);
    if (m->n_free < 1 || m->n_free > m->n_full)
        return fail(EMP_E_INVALID, "n_free=%d outside [1, n_full=%d]", m->n_free, m->n_full);
    if (m->n_planets < 0 || m->n_planets > EMP_MAX_PLANETS)
        return fail(EMP_E_SIZE, "n_planets=%d outside [0, %d]", m->n_planets, EMP_MAX_PLANETS);
    if (m->n_ins < 1 || m->n_ins > EMP_MAX_INS)
        return fail(EMP_E_SIZE, "n_ins=%d outside [1, %d]", m->n_ins, EMP_MAX_INS);
    if (m->ma_order < 0 || m->ma_order > EMP_MAX_MA)
        return fail(EMP_E_SIZE, "MA order %d outside [0, %d]", m->ma_order, EMP_MAX_MA);
    if (m->acc_order < 0 || m->acc_order > 8)
        return fail(EMP_E_SIZE, "acceleration order %d outside [0, 8]", m->acc_order);
    for (int p = 0; p < m->n_planets; ++p) {
        int par = m->kep_param[p];
        if (!(par == 0 || par == 1 || par == 2 || par == 3 || par == 4 || par == 6 || par == 7 ||
              par == EMP_TERM_SINUSOID || par == EMP_TERM_CYCLE_1 || par == EMP_TERM_CYCLE_2))
            return fail(EMP_E_UNSUPPORTED, "planet %d: parameterisation %d not built", p, par);
        const int nslot = par == EMP_TERM_SINUSOID ? 3 : 5;
        if (m->kep_slot[p] < 0 || m->kep_slot[p] + nslot > m->n_full)
            return fail(EMP_E_INVALID, "planet %d: slot %d out of range", p, m->kep_slot[p]);
        if (p > 0) {
            const int pp = m->kep_param[p - 1];
            // the two terms of a magnetic-cycle block share its slots
            const bool shared = par == EMP_TERM_CYCLE_2 && pp == EMP_TERM_CYCLE_1 &&
                                m->kep_slot[p] == m->kep_slot[p - 1];
            if (!shared && m->kep_slot[p] < m->kep_slot[p - 1] + (pp == EMP_TERM_SINUSOID ? 3 : 5))
                return fail(EMP_E_INVALID, "planet %d: slots overlap", p);
        }
        for (int k = 0; k < 2; ++k) {
            int rc = validate_prior(m->derived[p][k], "derived prior of planet", p);
            if (rc) return rc;
        }
    }
    auto chk = [&](int slot, int count, const char* nm) -> int {
        if (slot < 0) return EMP_OK;
        if (slot + count > m->n_full) return fail(EMP_E_INVALID, "%s slot %d + %d > n_full", nm, slot, count);
        return EMP_OK;
    };
    int rc;
    if ((rc = chk(m->offset_slot, m->n_ins, "offset"))) return rc;
    if ((rc = chk(m->jitter_slot, m->n_ins, "jitter"))) return rc;
    if ((rc = chk(m->acc_slot, m->acc_order, "acceleration"))) return rc;
    if (m->ma_order > 0) {
        if (m->ma_slot < 0) return fail(EMP_E_INVALID, "MA order > 0 without MA slot");
        int cnt = m->ma_global ? 2 * m->ma_order : 2 * m->ma_order * m->n_ins;
        if ((rc = chk(m->ma_slot, cnt, "MA"))) return rc;
    }
    if (m->acc_order > 0 && m->acc_slot < 0) return fail(EMP_E_INVALID, "acceleration without slot");
    if (m->hill_mask != 0) {
        if (m->hill_mask & ~(int)(((1u << (EMP_MAX_PLANETS + 1)) - 1u) & ~3u))
            return fail(EMP_E_INVALID, "hill_mask 0x%x names planet counts outside 2..%d", m->hill_mask,
                        EMP_MAX_PLANETS);
        int top = 0;
        for (int j = 2; j <= EMP_MAX_PLANETS; ++j)
            if (m->hill_mask & (1 << j)) top = j;
        if (top > m->n_planets)
            return fail(EMP_E_INVALID, "Hill prior over %d Keplerians, the model has %d terms", top, m->n_planets);
        if (!(m->hill_starmass > 0))
            return fail(EMP_E_INVALID, "Hill prior: star mass %g must be > 0", m->hill_starmass);
        for (int p = 0; p < top; ++p) {
            const int par = m->kep_param[p];
            if (!(par == 0 || par == 1 || par == 2 || par == 3 || par == 4 || par == 6))
                return fail(EMP_E_UNSUPPORTED, "Hill prior: term %d has parameterisation %d (0-4, 6 read "
                            "as the reference reads them)", p, par);
        }
    }
    if (m->am_on) {
        // every Keplerian an astrometric one: parameterisation 0 with inclination and node
        for (int p = 0; p < m->n_planets; ++p)
            if (m->kep_param[p] != 0 || m->kep_slot[p] + 7 > m->n_full)
                return fail(EMP_E_UNSUPPORTED, "astrometry: term %d is not a 7-slot parameterisation-0 Keplerian", p);
        if (m->am_offset_slot < 0 || m->am_jitter_slot < 0)
            return fail(EMP_E_INVALID, "astrometry without offset or jitter slots");
        if ((rc = chk(m->am_offset_slot, 5, "astrometric offset"))) return rc;
        if ((rc = chk(m->am_jitter_slot, 2, "astrometric jitter"))) return rc;
        if (m->gp_nterms > 0) return fail(EMP_E_UNSUPPORTED, "a GP likelihood with astrometry");
    }
    if (m->gp_nterms < 0 || m->gp_nterms > EMP_MAX_GP_TERMS)
        return fail(EMP_E_SIZE, "gp_nterms=%d outside [0, %d]", m->gp_nterms, EMP_MAX_GP_TERMS);
    if (m->gp_nterms > 0) {
        int dims = 0;
        for (int j = 0; j < m->gp_nterms; ++j) {
            const int kind = m->gp_kind[j];
            const int nd = gp_term_dims(kind);
            if (nd < 0) return fail(EMP_E_UNSUPPORTED, "GP term %d: kind %d unknown", j, kind);
            dims += nd;
            const int np = kind == EMP_GP_REAL || kind == EMP_GP_MATERN32 ? 2
                         : kind == EMP_GP_ROTATION ? 5 : kind == EMP_GP_GROT ? 4 : 3;
            for (int i = 0; i < 5; ++i) {
                const int sl = m->gp_slot[j][i];
                if (i < np && (sl < 0 || sl >= m->n_full))
                    return fail(EMP_E_INVALID, "GP term %d parameter %d: slot %d out of range", j, i, sl);
                if (i >= np && sl != -1)
                    return fail(EMP_E_INVALID, "GP term %d: slot %d of an unused parameter must be -1", j, i);
            }
        }
        if (dims > 16)
            return fail(EMP_E_UNSUPPORTED, "GP terms of %d state dimensions (at most 16)", dims);
    }
    std::vector<int> seen(m->n_free, 0);
    for (int s = 0; s < m->n_full; ++s) {
        int src = m->full_src[s];
        if (src >= m->n_free) return fail(EMP_E_INVALID, "full_src[%d]=%d >= n_free", s, src);
        if (src >= 0) seen[src]++;
        else if (!isfinite(m->full_fixed[s])) return fail(EMP_E_INVALID, "fixed value of slot %d not finite", s);
    }
    if (m->n_prior_var < 0 || m->n_prior_var > m->n_free + 2 * m->n_planets)
        return fail(EMP_E_INVALID, "n_prior_var=%d out of range", m->n_prior_var);
    for (int i = 0; i < m->n_prior_var; ++i) {
        const int v = m->prior_var[i];
        if (v < 0 || v >= m->n_free + 2 * m->n_planets)
            return fail(EMP_E_INVALID, "prior_var[%d]=%d out of range", i, v);
        const emp_prior& p = v < m->n_free ? m->prior[v] : m->derived[(v - m->n_free) >> 1][(v - m->n_free) & 1];
        if (p.kind != EMP_PRIOR_NORMAL && p.kind != EMP_PRIOR_BETA && p.kind != EMP_PRIOR_ISOTROPIC)
            return fail(EMP_E_INVALID, "prior_var[%d] names a constant prior", i);
    }
    for (int i = 0; i < m->n_free; ++i) {
        if (seen[i] != 1) return fail(EMP_E_INVALID, "free parameter %d mapped %d times", i, seen[i]);
        int sl = m->prior_slot[i];
        if (sl < 0 || sl >= m->n_full || m->full_src[sl] != i)
            return fail(EMP_E_INVALID, "prior_slot[%d]=%d inconsistent with full_src", i, sl);
        if (i > 0 && sl <= m->prior_slot[i - 1]) return fail(EMP_E_INVALID, "prior_slot not increasing");
        if ((rc = validate_prior(m->prior[i], "prior of free parameter", i))) return rc;
        if (m->prior[i].kind == EMP_PRIOR_NONE)
            return fail(EMP_E_INVALID, "free parameter %d has no prior", i);
    }
    return EMP_OK;
}

// default lanes per walker when the autotuner has not set one: about 16
// epochs per lane for the mixed kernel (measured best for N=1024 at 1280
// walkers), more lanes for the FP64 kernel, whose per-epoch work is longer
int pick_default_L(int prec, int n) {
    int target = prec == EMP_PREC_FP64 ? n / 8 : n / 16;
    int L = 8;
    while (L < target && L < (prec == EMP_PREC_FP64 ? 128 : 64)) L <<= 1;
    return L;
}

int pick_tile(const emp_handle* h, int prec, int L, int G, Smem& lay) {
    int want = h->tile[prec];
    if (want <= 0) want = prec == EMP_PREC_FP64 ? 1024 : 2048;
    // the lane-chunk layout of a tile of nt epochs occupies ceil(nt/L)*L
    // slots, so the tile is a multiple of L
    auto round_L = [L](int x) { return ((x + L - 1) / L) * L; };
    int t = round_L(std::min(want, h->n));
    t = std::max(t, L);
    for (;;) {
        lay.build(prec, h->q, L, G, t, h->lay[0], h->lay[1], h->lay[2], h->lay[3], h->lay[4],
                  (h->gp_M > 0 && h->q > 0) ? 1 : 0);
        if (lay.total <= 200 * 1024 || t <= L) break;
        t = std::max(L, round_L(t / 2));
    }
    return t;
}

int handle_L(const emp_handle* h, int prec) {
    return h->L[prec] > 0 ? h->L[prec] : pick_default_L(prec, h->n_typ);
}

// Kernel attributes (and, for a batch, the persistent grid) set up outside
// any stream capture.
int prepare_eval(emp_handle* h, int prec) {
    const int L = handle_L(h, prec);
    const int li = lanes_index(L);
    if (li < 0) return fail(EMP_E_INVALID, "lanes per walker %d not built", L);
    KFn fn = prec == EMP_PREC_FP64 ? get_kernel_fp64(h->q, li) : get_kernel_mixed(h->q, li);
    if (!fn) return fail(EMP_E_UNSUPPORTED, "no kernel for q=%d L=%d", h->q, L);
    if (!h->attr_done[prec][h->q][li]) {
        // 227 KB per block covers the static shared memory too
        cudaFuncAttributes fa;
        CUDA_TRY(cudaFuncGetAttributes(&fa, (const void*)fn));
        CUDA_TRY(cudaFuncSetAttribute((const void*)fn, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                      227 * 1024 - (int)fa.sharedSizeBytes));
        h->attr_done[prec][h->q][li] = true;
    }
    if (h->n_sys > 1) {
        const int NT = L > 128 ? L : 128;
        Smem lay;
        pick_tile(h, prec, L, NT / L, lay);
        if (h->persist_smem[prec][li] != lay.total || h->persist_grid[prec][li] <= 0) {
            int dev = 0, sms = 0, nb = 0;
            CUDA_TRY(cudaGetDevice(&dev));
            CUDA_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
            CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, (const void*)fn, NT, lay.total));
            h->persist_grid[prec][li] = std::max(1, nb) * sms;
            h->persist_smem[prec][li] = lay.total;
        }
    }
    return EMP_OK;
}

// Everything a sweep sets up on the device once per handle (the stretch
// kernel's attributes and persistent grid, the swap kernel's shared-memory
// limit), done before the sweep's first launch.
int prepare_sweep(emp_handle* h, int prec) {
    int rc = prepare_eval(h, prec);
    if (rc) return rc;
    if (!h->swap_attr) {
        CUDA_TRY(cudaFuncSetAttribute((const void*)k_swap<true, false>,
                                      cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kSwapSmemMax));
        CUDA_TRY(cudaFuncSetAttribute((const void*)k_swap<true, false, true>,
                                      cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kSwapSmemMax));
        h->swap_attr = true;
    }
    if (!h->swap_attr_batch) {
        CUDA_TRY(cudaFuncSetAttribute((const void*)k_swap<true, true>,
                                      cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kSwapSmemMax));
        h->swap_attr_batch = true;
    }
    return EMP_OK;
}

void gp_args(const emp_handle* h, KArgs& a);
int launch_gp(emp_handle* h, KArgs& a, cudaStream_t s, int prec);

// a launch that may overlap the previous kernel of the stream (programmatic
// dependent launch): the kernel starts once every CTA of the previous one
// runs and executes griddepcontrol.wait before reading its results
template <typename Arg>
cudaError_t launch_pdl(void (*fn)(Arg), dim3 grid, dim3 block, size_t smem, cudaStream_t s, Arg arg) {
    cudaLaunchConfig_t cfg{};
    cfg.gridDim = grid;
    cfg.blockDim = block;
    cfg.dynamicSmemBytes = smem;
    cfg.stream = s;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    return cudaLaunchKernelEx(&cfg, fn, arg);
}

// counter: for a batch, the int that CTAs of a persistent launch claim
// items from (zeroed here, in stream order); null launches one CTA per item
int launch_eval(emp_handle* h, int prec, KArgs& a, cudaStream_t s, unsigned* counter = nullptr,
                bool pdl = false) {
    if (prec != EMP_PREC_FP64 && prec != EMP_PREC_MIXED)
        return fail(EMP_E_INVALID, "precision %d unknown", prec);
    int L = handle_L(h, prec);
    int li = lanes_index(L);
    if (li < 0) return fail(EMP_E_INVALID, "lanes per walker %d not built", L);
    int NT = L > 128 ? L : 128;
    int G = NT / L;
    Smem lay;
    int tile = pick_tile(h, prec, L, G, lay);
    if (lay.total > 227 * 1024 - 64)
        return fail(EMP_E_SIZE, "shared memory %d B exceeds 227 KB", lay.total);
    KFn fn = prec == EMP_PREC_FP64 ? get_kernel_fp64(h->q, li) : get_kernel_mixed(h->q, li);
    if (!fn) return fail(EMP_E_UNSUPPORTED, "no kernel for q=%d L=%d", h->q, L);
    if (!h->attr_done[prec][h->q][li] || (h->n_sys > 1 && h->persist_smem[prec][li] != lay.total)) {
        int rc = prepare_eval(h, prec);
        if (rc) return rc;
    }
    a.md = h->md_dev;
    a.d = h->dd;
    a.tile = tile;
    a.lay_full = h->lay[0];
    a.lay_free = h->lay[1];
    a.lay_planets = h->lay[2];
    a.lay_ins = h->lay[3];
    a.lay_acc = h->lay[4];
    a.dstride = h->lay[1];
    a.n_sys = h->n_sys;
    a.sys_off = h->sys_off;
    a.sys_t0 = h->sys_t0;
    a.sys_order = h->sys_order;
    if (a.nwalk <= 0) return EMP_OK;
    bool gp = false;
    if (h->gp_M > 0) {
        if (a.nwalk > h->gp_rows)
            return fail(EMP_E_INVALID, "GP workspace holds %lld rows, launch has %d", (long long)h->gp_rows, a.nwalk);
        gp = true;
        gp_args(h, a);
    }
    const bool am = h->md.am_on != 0;
    if (am) {
        if (!h->am_set) return fail(EMP_E_INVALID, "the model has astrometry but emp_set_astrometry was not called");
        a.am = h->am;
        a.am_sys = h->am_sys;
        if (a.mode == kModeStretch) {
            if (a.nwalk > h->am_rows)
                return fail(EMP_E_INVALID, "astrometry rows hold %lld walkers, launch has %d", (long long)h->am_rows,
                            a.nwalk);
            a.am_rv = h->am_rv;
            a.gp_meta = h->am_meta;
            a.gp_prop = h->am_prop;
        }
    }
    a.cps = (a.nwalk + G - 1) / G;
    const int64_t items = (int64_t)a.cps * h->n_sys;
    if (items > 0x7fffffff) return fail(EMP_E_SIZE, "%lld CTA items exceed 2^31-1", (long long)items);
    int grid = (int)items;
    a.work_counter = nullptr;
    if (counter != nullptr && h->n_sys > 1) {
        a.work_counter = reinterpret_cast<int*>(counter);
        grid = (int)std::min<int64_t>(items, h->persist_grid[prec][li]);
        CUDA_TRY(cudaMemsetAsync(counter, 0, sizeof(unsigned), s));
    }
    if (pdl) CUDA_TRY(launch_pdl(fn, dim3(grid), dim3(NT), (size_t)lay.total, s, a));
    else fn<<<grid, NT, lay.total, s>>>(a);
    g_launches.fetch_add(1);
    CUDA_TRY(cudaGetLastError());
    if (gp) return launch_gp(h, a, s, prec);
    if (am) {
        const int rows_per_cta = kAmThreads / 32;
        get_kernel_am(prec)<<<dim3((unsigned)((a.nwalk + rows_per_cta - 1) / rows_per_cta), (unsigned)h->n_sys),
                          kAmThreads, 0, s>>>(a);
        g_launches.fetch_add(1);
        CUDA_TRY(cudaGetLastError());
    }
    return EMP_OK;
}

// Stretch buffers of the astrometric term for up to `rows` walker rows per
// system (proposal, meta, RV logL; [systems][rows]); allocated outside any
// capture, growing drops the captured sweep graphs.
int am_reserve(emp_handle* h, int64_t rows) {
    if (!h->md.am_on || rows <= h->am_rows) return EMP_OK;
    const size_t D = (size_t)std::max(h->lay[1], 1), R = (size_t)rows * (size_t)h->n_sys;
    auto up = [](size_t b) { return (b + 255) & ~(size_t)255; };
    const size_t b_prop = up(8 * D * R), b_meta = up(sizeof(GPMeta) * R);
    const size_t b_rv = up(8 * R);
    h->gc.reset();
    h->gch.reset();
    if (h->am_rows_buf) {
        cudaFree(h->am_rows_buf);
        h->am_rows_buf = nullptr;
        h->am_rows = 0;
    }
    void* b = nullptr;
    CUDA_TRY(cudaMalloc(&b, b_prop + b_meta + b_rv));
    unsigned char* c = (unsigned char*)b;
    h->am_rows_buf = b;
    h->am_prop = (double*)c;
    h->am_meta = (GPMeta*)(c + b_prop);
    h->am_rv = (double*)(c + b_prop + b_meta);
    h->am_rows = rows;
    return EMP_OK;
}

// GP row buffers for launches of up to `rows` walker rows per system;
// allocated (or grown) outside any stream capture, before the launches that
// use them.  A captured sweep graph refers to the old buffers, so growing
// drops it.  Epoch-major arrays are [all systems' epochs][rows] (system s
// from its first epoch on), row arrays [systems][rows].
int gp_reserve(emp_handle* h, int64_t rows) {
    if (h->gp_M == 0 || rows <= h->gp_rows) return EMP_OK;
    const size_t n = (size_t)h->dd.n, D = (size_t)std::max(h->lay[1], 1), S = (size_t)h->n_sys;
    const size_t al = 256;
    auto up = [al](size_t b) { return (b + al - 1) & ~(al - 1); };
    const size_t b_re = up(8 * n * (size_t)rows);
    const size_t b_prop = up(8 * D * (size_t)rows * S);
    const size_t b_meta = up(sizeof(GPMeta) * (size_t)rows * S);
    const size_t b_uvp = up(8 * n * (size_t)rows * (size_t)h->gp_M);
    const size_t b_asum = up(8 * (size_t)rows * S);
    const size_t total = 2 * b_re + b_prop + b_meta + 3 * b_uvp + b_asum;
    if (total > ((size_t)64 << 30))
        return fail(EMP_E_SIZE, "GP workspace of %zu B for %lld rows exceeds 64 GiB", total, (long long)rows);
    h->gc.reset();
    h->gch.reset();
    if (h->gp_buf) {
        cudaFree(h->gp_buf);
        h->gp_buf = nullptr;
        h->gp_rows = 0;
    }
    void* b = nullptr;
    CUDA_TRY(cudaMalloc(&b, total));
    unsigned char* c = (unsigned char*)b;
    h->gp_buf = b;
    h->gp_r = (double*)c;
    h->gp_e = (double*)(c + b_re);
    h->gp_prop = (double*)(c + 2 * b_re);
    h->gp_meta = (GPMeta*)(c + 2 * b_re + b_prop);
    unsigned char* c2 = c + 2 * b_re + b_prop + b_meta;
    h->gp_u = (double*)c2;
    h->gp_v = (double*)(c2 + b_uvp);
    h->gp_ph = (double*)(c2 + 2 * b_uvp);
    h->gp_asum = (double*)(c2 + 3 * b_uvp);
    if (h->sms <= 0) {
        int dev = 0;
        CUDA_TRY(cudaGetDevice(&dev));
        CUDA_TRY(cudaDeviceGetAttribute(&h->sms, cudaDevAttrMultiProcessorCount, dev));
    }
    h->gp_rows = rows;
    return EMP_OK;
}

void gp_args(const emp_handle* h, KArgs& a) {
    a.gp_r = h->gp_r;
    a.gp_e = h->gp_e;
    a.gp_prop = h->gp_prop;
    a.gp_meta = h->gp_meta;
    a.gp_u = h->gp_u;
    a.gp_v = h->gp_v;
    a.gp_ph = h->gp_ph;
    a.gp_asum = h->gp_asum;
}

// The GP likelihood of the rows of `a`: k_gp_prep (every row x epoch, about
// 16 warps per SM) then the FP64 recursion k_gp (M lanes per row), or for
// the mixed precision k_gp_fused (both in one kernel, float-float); the
// last grid dimension is the system of a batch handle
int launch_gp(emp_handle* h, KArgs& a, cudaStream_t s, int prec) {
    const int M = h->gp_M;
    const int ff = prec == EMP_PREC_MIXED ? 1 : 0;
    if (ff) {
        // preparation and recursion in one kernel: a CTA per 32/M rows (one
        // warp of the recursion, kGPProducers warps preparing its inputs)
        KFn fused = get_kernel_gp(M, 0, 1);
        if (!fused) return fail(EMP_E_UNSUPPORTED, "no GP kernel for %d state dimensions", M);
        const int R = 32 / M;
        fused<<<dim3((unsigned)((a.nwalk + R - 1) / R), (unsigned)h->n_sys), 32 * (1 + kGPProducers), 0, s>>>(a);
        g_launches.fetch_add(1);
        CUDA_TRY(cudaGetLastError());
        return EMP_OK;
    }
    KFn prep = get_kernel_gp(M, 1, ff), rec = get_kernel_gp(M, 0, ff);
    if (!prep || !rec) return fail(EMP_E_UNSUPPORTED, "no GP kernel for %d state dimensions", M);
    const int gx = (a.nwalk + 31) / 32;
    const int want_warps = std::max(1, h->sms) * 16;
    const int64_t per_y = 8 * (int64_t)gx * h->n_sys;
    const int gy = (int)std::max<int64_t>(1, std::min<int64_t>((h->n + 7) / 8, (want_warps + per_y - 1) / per_y));
    prep<<<dim3(gx, gy, (unsigned)h->n_sys), 256, 0, s>>>(a);
    g_launches.fetch_add(1);
    CUDA_TRY(cudaGetLastError());
    const int64_t threads = (int64_t)a.nwalk * M;
    rec<<<dim3((unsigned)((threads + kGPBlock - 1) / kGPBlock), (unsigned)h->n_sys), kGPBlock, 0, s>>>(a);
    g_launches.fetch_add(1);
    CUDA_TRY(cudaGetLastError());
    return EMP_OK;
}

int check_state(const emp_handle* h, const emp_pt_state* st) {
    if (!st) return fail(EMP_E_INVALID, "state is NULL");
    if (st->ntemps < 1 || st->ntemps > kMaxTemps)
        return fail(EMP_E_SIZE, "ntemps=%d outside [1, %d]", st->ntemps, kMaxTemps);
    if (st->nwalkers < 2 || (st->nwalkers & 1))
        return fail(EMP_E_INVALID, "nwalkers=%d must be even and >= 2", st->nwalkers);
    if (st->nwalkers > 65534) return fail(EMP_E_SIZE, "nwalkers=%d exceeds 65534", st->nwalkers);
    const int nsys = st->n_systems <= 0 ? 1 : st->n_systems;
    if (nsys != h->n_sys)
        return fail(EMP_E_INVALID, "state holds %d systems, handle %d", nsys, h->n_sys);
    if ((int64_t)nsys * st->ntemps * st->nwalkers > 0x7fffffff)
        return fail(EMP_E_SIZE, "systems*ntemps*nwalkers exceeds 2^31-1");
    if (st->ndim != h->lay[1])
        return fail(EMP_E_INVALID, "state ndim=%d but the model%s %d free parameters", st->ndim,
                    h->n_sys > 1 ? "s' largest free dimension is" : " has", h->lay[1]);
    if (st->nsteps < 1) return fail(EMP_E_INVALID, "nsteps=%d < 1", st->nsteps);
    if (!st->theta || !st->logl || !st->logprior || !st->members || !st->betas || !st->counters ||
        !st->accepted || !st->swaps_accepted || !st->perm_units)
        return fail(EMP_E_INVALID, "a state buffer is NULL");
    if (st->n_perm_units < 1) return fail(EMP_E_INVALID, "no permutation units");
    if (st->precision != EMP_PREC_FP64 && st->precision != EMP_PREC_MIXED)
        return fail(EMP_E_INVALID, "precision %d unknown", st->precision);
    if (st->adapt && st->adapt_mode != 0)
        return fail(EMP_E_UNSUPPORTED, "adapt_mode %d not built (0 is)", st->adapt_mode);
    if (!(st->a > 1.0)) return fail(EMP_E_INVALID, "stretch scale a=%g must be > 1", st->a);
    if (st->adapt && !(st->adapt_tau > 0 && st->adapt_nu > 0))
        return fail(EMP_E_INVALID, "adapt_tau and adapt_nu must be > 0");
    if (!st->work) return fail(EMP_E_INVALID, "state workspace is NULL");
    if (st->work_bytes < (int64_t)work_bytes(st->ntemps, st->nwalkers))
        return fail(EMP_E_SIZE, "workspace of %lld B < %zu B needed", (long long)st->work_bytes,
                    work_bytes(st->ntemps, st->nwalkers));
    if (((uintptr_t)st->work) & 15) return fail(EMP_E_INVALID, "workspace not 16-byte aligned");
    return EMP_OK;
}

// copy of the packed walker state back to the host, overlapped with the swap
// and record kernels (emp_pt_run_host)
struct HostCopy {
    void* host;
    size_t bytes;
    cudaStream_t aux;
    cudaEvent_t ev[2];
};

int enqueue_sweep(emp_handle* h, const emp_pt_state* st, const emp_pt_record* rec,
                  cudaStream_t s, int* nkern, const HostCopy* hc = nullptr) {
    int rc;
    int kcount = 0;
    const bool batch = h->n_sys > 1;
    Work work = carve_work(st->work);
    for (int step = 0; step < st->nsteps; ++step) {
        for (int half = 0; half < 2; ++half) {
            KArgs a{};
            a.mode = kModeStretch;
            a.nwalk = st->ntemps * (st->nwalkers / 2);
            a.st_theta = st->theta;
            a.st_logl = st->logl;
            a.st_logprior = st->logprior;
            a.members = st->members;
            a.betas = st->betas;
            a.counters = st->counters;
            a.accepted = st->accepted;
            a.W = st->nwalkers;
            a.T = st->ntemps;
            a.half = half;
            a.step_in_sweep = step;
            a.seed = st->seed;
            a.a = st->a;
            {
                int ex = 0;
                a.a_inv_exact = frexp(st->a, &ex) == 0.5 ? 1.0 / st->a : 0.0;   // a = 2^(ex-1)
            }
            if ((rc = launch_eval(h, st->precision, a, s, batch ? work.ticket + 1 : nullptr, !batch))) return rc;
            kcount += h->gp_M > 0 ? (st->precision == EMP_PREC_MIXED ? 2 : 3) : (h->md.am_on ? 2 : 1);
        }
    }
    if (hc) {
        // the walker state is final after the stretch moves (the swaps
        // exchange slot ids, the record only reads it): copy it back on a
        // second stream while the swap and record kernels run
        CUDA_TRY(cudaEventRecord(hc->ev[0], s));
        CUDA_TRY(cudaStreamWaitEvent(hc->aux, hc->ev[0], 0));
        CUDA_TRY(cudaMemcpyAsync(hc->host, st->theta, hc->bytes, cudaMemcpyDeviceToHost, hc->aux));
        CUDA_TRY(cudaEventRecord(hc->ev[1], hc->aux));
    }
    SwapArgs S{};
    S.T = st->ntemps; S.W = st->nwalkers; S.D = st->ndim; S.nsteps = st->nsteps;
    S.n_sys = h->n_sys;
    S.logl = st->logl; S.members = st->members; S.betas = st->betas;
    S.counters = st->counters; S.swaps_accepted = st->swaps_accepted;
    S.units = st->perm_units; S.nunits = st->n_perm_units;
    S.adapt = st->adapt; S.adapt_mode = st->adapt_mode;
    S.adapt_tau = st->adapt_tau; S.adapt_nu = st->adapt_nu; S.seed = st->seed;
    S.work = work;
    const bool have_rec = rec && rec->n_recorded;
    S.beta_hist = have_rec ? rec->beta_history : nullptr;
    S.tsw_hist = have_rec ? rec->tsw_history : nullptr;
    S.have_smd = have_rec && rec->smd_history != nullptr;
    S.n_rec = have_rec ? rec->n_recorded : S.work.nrec_none;
    S.cap = have_rec ? rec->capacity : 0;
    S.thin = have_rec ? std::max(1, rec->thin) : 1;
    S.record_chain = have_rec && (rec->chain || rec->log_like || rec->log_prob);
    S.theta = st->theta;
    S.logprior = st->logprior;
    S.chain = have_rec ? rec->chain : nullptr;
    S.log_like = have_rec ? rec->log_like : nullptr;
    S.log_prob = have_rec ? rec->log_prob : nullptr;
    S.smd_hist = have_rec ? rec->smd_history : nullptr;
    const size_t swap_smem = (size_t)st->ntemps * st->nwalkers * 24;
    if (batch) {
        // one CTA per system; threads cover a temperature's walkers
        const int nthb = std::min(1024, std::max(128, (st->nwalkers + 31) / 32 * 32));
        if (swap_smem <= kSwapSmemMax) {
            if (!h->swap_attr_batch) {
                CUDA_TRY(cudaFuncSetAttribute((const void*)k_swap<true, true>,
                                              cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kSwapSmemMax));
                h->swap_attr_batch = true;
            }
            k_swap<true, true><<<h->n_sys, nthb, swap_smem, s>>>(S);
        } else {
            k_swap<false, true><<<h->n_sys, nthb, 0, s>>>(S);
        }
        g_launches.fetch_add(1);
        ++kcount;
        CUDA_TRY(cudaGetLastError());
        if (S.record_chain) {
            RecBatchArgs R{};
            R.S = h->n_sys; R.T = st->ntemps; R.W = st->nwalkers; R.D = st->ndim;
            R.theta = st->theta; R.logl = st->logl; R.logprior = st->logprior;
            R.members = st->members; R.betas = st->betas; R.counters = st->counters;
            R.n_rec = S.n_rec; R.cap = S.cap; R.thin = S.thin;
            R.chain = rec->chain; R.log_like = rec->log_like; R.log_prob = rec->log_prob;
            const int64_t tot = (int64_t)h->n_sys * st->nwalkers * (rec->chain ? st->ndim : 1);
            const int grid = (int)std::min<int64_t>(std::max<int64_t>(1, (tot + 255) / 256), 152 * 8);
            k_record_batch<<<grid, 256, 0, s>>>(R);
            g_launches.fetch_add(1);
            ++kcount;
            CUDA_TRY(cudaGetLastError());
        }
        AdvArgs V{};
        V.counters = st->counters; V.n_rec = S.n_rec; V.cap = S.cap; V.thin = S.thin;
        V.nsteps = st->nsteps; V.record_chain = S.record_chain;
        k_advance<<<1, 32, 0, s>>>(V);
        g_launches.fetch_add(1);
        ++kcount;
        CUDA_TRY(cudaGetLastError());
        if (nkern) *nkern = kcount;
        return EMP_OK;
    }
    const int nth = 1024;
    // small history rows are written by the swap CTA itself (one launch less)
    const size_t rec_bytes = (size_t)st->ntemps * st->nwalkers * (size_t)(st->ndim + 2) * 8;
    const bool rec_in_swap = swap_smem <= kSwapSmemMax && rec_bytes <= kRecInSwapMax;
    if (swap_smem <= kSwapSmemMax) {
        if (!h->swap_attr) {
            CUDA_TRY(cudaFuncSetAttribute((const void*)k_swap<true, false>,
                                          cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kSwapSmemMax));
            CUDA_TRY(cudaFuncSetAttribute((const void*)k_swap<true, false, true>,
                                          cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kSwapSmemMax));
            h->swap_attr = true;
        }
        if (rec_in_swap) CUDA_TRY(launch_pdl(k_swap<true, false, true>, dim3(1), dim3(nth), swap_smem, s, S));
        else CUDA_TRY(launch_pdl(k_swap<true, false>, dim3(1), dim3(nth), swap_smem, s, S));
    } else {
        CUDA_TRY(launch_pdl(k_swap<false, false>, dim3(1), dim3(nth), (size_t)0, s, S));
    }
    g_launches.fetch_add(1);
    ++kcount;
    CUDA_TRY(cudaGetLastError());
    if ((S.record_chain || S.have_smd) && !rec_in_swap) {
        RecArgs R{};
        R.T = st->ntemps; R.W = st->nwalkers; R.D = st->ndim;
        R.theta = st->theta; R.logl = st->logl; R.logprior = st->logprior;
        R.members = st->members; R.work = S.work;
        R.chain = rec->chain; R.log_like = rec->log_like; R.log_prob = rec->log_prob;
        R.smd_hist = rec->smd_history;
        const int64_t tot = (int64_t)st->ntemps * st->nwalkers * (rec->chain ? st->ndim : 1);
        const int64_t warps = (int64_t)(st->ntemps - 1) * st->nwalkers;
        const int64_t want = std::max((tot + 255) / 256, (warps + 7) / 8);
        const int grid = (int)std::min<int64_t>(std::max<int64_t>(1, want), 152 * 8);
        CUDA_TRY(launch_pdl(k_record, dim3(grid), dim3(256), (size_t)0, s, R));
        g_launches.fetch_add(1);
        ++kcount;
        CUDA_TRY(cudaGetLastError());
    }
    if (hc) CUDA_TRY(cudaStreamWaitEvent(s, hc->ev[1], 0));    // join the copy back
    if (nkern) *nkern = kcount;
    return EMP_OK;
}

bool same_state(const emp_pt_state& a, const emp_pt_state& b) {
    return memcmp(&a, &b, sizeof(a)) == 0;
}
bool same_rec(const emp_pt_record& a, const emp_pt_record& b) {
    return memcmp(&a, &b, sizeof(a)) == 0;
}

}  // namespace

namespace emp {
// error reporting for the other translation units (same last-error string)
int stats_fail(int code, const char* msg) { return fail(code, "%s", msg); }
void count_launch() { g_launches.fetch_add(1); }
}  // namespace emp

extern "C" {

int emp_abi_version(void) { return EMP_ABI_VERSION; }

const char* emp_last_error_string(void) { return g_err; }

int64_t emp_launch_count(void) { return g_launches.load(); }

}  // extern "C"

namespace {

// Host preprocessing of one system's epochs into the device layout: time
// order, or instrument-grouped time order when each instrument carries its
// own MA series; squared errors; the FP32 hi/lo split of the times; the lag
// distances of the MA recurrence (+inf across a series start).
struct HostData {
    std::vector<double> t, y, s2, dt;
    std::vector<float> t_hi, t_lo, y32, y_lo, s2_32, dt32;
    std::vector<int> inst, orig;
    void reserve(size_t n, int q) {
        t.reserve(n); y.reserve(n); s2.reserve(n); t_hi.reserve(n); t_lo.reserve(n);
        y32.reserve(n); y_lo.reserve(n); s2_32.reserve(n); inst.reserve(n); orig.reserve(n);
        (void)q;
    }
};

int check_system(const emp_model_desc* model, const emp_dataset_desc* data, int s, int64_t* n_out) {
    const int64_t n64 = data->offsets[s + 1] - data->offsets[s];
    if (n64 <= 0) return fail(EMP_E_INVALID, "system %d has %lld epochs", s, (long long)n64);
    if (n64 > (1 << 26)) return fail(EMP_E_SIZE, "system %d: %lld epochs exceed 2^26", s, (long long)n64);
    const int64_t o = data->offsets[s];
    const double* t = data->t + o;
    const double* y = data->y + o;
    const double* ye = data->yerr + o;
    const int32_t* in = data->inst + o;
    for (int64_t i = 0; i < n64; ++i) {
        if (!isfinite(t[i]) || !isfinite(y[i]) || !isfinite(ye[i]))
            return fail(EMP_E_INVALID, "system %d epoch %lld has a non-finite value", s, (long long)i);
        if (in[i] < 1 || in[i] > model->n_ins)
            return fail(EMP_E_INVALID, "system %d epoch %lld: instrument %d outside 1..%d", s, (long long)i,
                        in[i], model->n_ins);
        if (i > 0 && t[i] < t[i - 1])
            return fail(EMP_E_INVALID, "system %d: times not sorted at epoch %lld", s, (long long)i);
    }
    *n_out = n64;
    return EMP_OK;
}

int ma_order_on_device(const emp_model_desc* m) {
    const bool ma_on = m->ma_order > 0 && (m->ma_global || !m->ma_quirk);
    return ma_on ? m->ma_order : 0;
}

void append_system(const emp_model_desc* model, const emp_dataset_desc* data, int s, int q,
                   HostData& H, std::vector<std::vector<double>>& dts) {
    const int64_t o = data->offsets[s];
    const int n = (int)(data->offsets[s + 1] - o);
    const double* t = data->t + o;
    const double* y = data->y + o;
    const double* ye = data->yerr + o;
    const int32_t* in = data->inst + o;
    const bool group_by_ins = q > 0 && !model->ma_global;
    std::vector<int> order(n);
    std::iota(order.begin(), order.end(), 0);
    if (group_by_ins)
        std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return in[a] < in[b]; });
    const size_t base = H.t.size();
    for (int i = 0; i < n; ++i) {
        const int k = order[i];
        H.t.push_back(t[k]);
        H.y.push_back(y[k]);
        H.s2.push_back(ye[k] * ye[k]);
        H.inst.push_back(in[k] - 1);
        const float hi = (float)t[k];
        H.t_hi.push_back(hi);
        H.t_lo.push_back((float)(t[k] - (double)hi));
        H.y32.push_back((float)y[k]);
        H.y_lo.push_back((float)(y[k] - (double)(float)y[k]));
        H.s2_32.push_back((float)(ye[k] * ye[k]));
        H.orig.push_back(k);
    }
    for (int c = 0; c < q; ++c) {
        for (int i = 0; i < n; ++i) {
            // predecessor at lag c+1 inside the same series (instrument or global)
            const int lag = c + 1;
            double v = INFINITY;
            if (i - lag >= 0 && (!group_by_ins || H.inst[base + i - lag] == H.inst[base + i]))
                v = fabs(H.t[base + i] - H.t[base + i - lag]);
            dts[c].push_back(v);
        }
    }
}

int create_impl(const emp_model_desc* models, int S, const emp_dataset_desc* data, emp_handle** out) {
    if (!out) return fail(EMP_E_INVALID, "out is NULL");
    *out = nullptr;
    if (!models) return fail(EMP_E_INVALID, "model descriptor is NULL");
    if (!data) return fail(EMP_E_INVALID, "dataset descriptor is NULL");
    if (!data->offsets || !data->t || !data->y || !data->yerr || !data->inst)
        return fail(EMP_E_INVALID, "a dataset array is NULL");
    int rc;
    const int q = ma_order_on_device(&models[0]);
    std::vector<int64_t> nsys(S);
    int64_t total = 0;
    int lay[5] = {0, 0, 0, 0, 0};
    for (int s = 0; s < S; ++s) {
        const emp_model_desc* m = &models[s];
        if ((rc = validate_model(m))) {
            if (S > 1) {
                char tmp[600];
                snprintf(tmp, sizeof(tmp), "system %d: %s", s, g_err);
                return fail(rc, "%s", tmp);
            }
            return rc;
        }
        if (ma_order_on_device(m) != q)
            return fail(EMP_E_UNSUPPORTED, "system %d: MA order %d differs from system 0's %d", s,
                        ma_order_on_device(m), q);
        if ((rc = check_system(m, data, s, &nsys[s]))) return rc;
        if ((m->am_on != 0) != (models[0].am_on != 0))
            return fail(EMP_E_UNSUPPORTED, "system %d: astrometric and RV-only systems in one batch", s);
        total += nsys[s];
        lay[0] = std::max(lay[0], m->n_full);
        lay[1] = std::max(lay[1], m->n_free);
        lay[2] = std::max(lay[2], m->n_planets);
        lay[3] = std::max(lay[3], m->n_ins);
        lay[4] = std::max(lay[4], m->acc_order);
    }
    if (total > (1 << 30)) return fail(EMP_E_SIZE, "%lld epochs in total exceed 2^30", (long long)total);
    const int n = (int)total;

    HostData H;
    H.reserve((size_t)n, q);
    std::vector<std::vector<double>> dts(std::max(q, 1));
    std::vector<int64_t> off(S + 1, 0);
    std::vector<double> t0(S);
    for (int s = 0; s < S; ++s) {
        off[s] = (int64_t)H.t.size();
        t0[s] = data->t[data->offsets[s]];
        append_system(&models[s], data, s, q, H, dts);
    }
    off[S] = (int64_t)H.t.size();
    const size_t qn = (size_t)std::max(q, 1) * n;
    std::vector<double> hdt(qn, INFINITY);
    std::vector<float> dtf(qn, INFINITY);
    for (int c = 0; c < q; ++c)
        for (int i = 0; i < n; ++i) {
            hdt[(size_t)c * n + i] = dts[c][i];
            dtf[(size_t)c * n + i] = (float)dts[c][i];
        }
    // costliest systems first: epochs x (planets + 1)
    std::vector<int> sorder(S);
    std::iota(sorder.begin(), sorder.end(), 0);
    std::stable_sort(sorder.begin(), sorder.end(), [&](int a, int b) {
        return nsys[a] * (models[a].n_planets + 1) > nsys[b] * (models[b].n_planets + 1);
    });
    std::vector<int64_t> sorted_n(nsys);
    std::sort(sorted_n.begin(), sorted_n.end());

    // one GP state dimension for every system of a batch: the largest, as a
    // power of two (a system's unused dimensions stay zero and add nothing;
    // a system without GP terms then has the Gaussian likelihood)
    int gp_M = 0;
    {
        int dims = 0;
        bool any = false;
        for (int s = 0; s < S; ++s) {
            int d = 0;
            for (int j = 0; j < models[s].gp_nterms; ++j) d += gp_term_dims(models[s].gp_kind[j]);
            dims = std::max(dims, d);
            any = any || models[s].gp_nterms > 0;
        }
        if (any) {
            gp_M = 2;
            while (gp_M < dims) gp_M <<= 1;
            if (S > 65535) return fail(EMP_E_SIZE, "%d systems with GP likelihoods (at most 65535)", S);
        }
    }
    if (models[0].am_on && S > 65535) return fail(EMP_E_SIZE, "%d systems with astrometry (at most 65535)", S);

    emp_handle* h = new (std::nothrow) emp_handle();
    if (!h) return fail(EMP_E_INVALID, "out of host memory");
    h->md = models[0];
    h->n = (int)sorted_n.back();
    h->n_typ = (int)sorted_n[S / 2];
    h->n_sys = S;
    for (int k = 0; k < 5; ++k) h->lay[k] = lay[k];
    h->q = q;
    if (gp_M > 0) h->gp_M = gp_M;

    // one device allocation for the dataset, descriptors and system tables
    size_t bytes = 0;
    auto take = [&](size_t b) { size_t o = bytes; bytes += (b + 255) & ~(size_t)255; return o; };
    const size_t N8 = 8 * (size_t)n, N4 = 4 * (size_t)n;
    size_t o_t = take(N8), o_y = take(N8), o_s2 = take(N8), o_dt = take(8 * qn);
    size_t o_th = take(N4), o_tl = take(N4), o_yf = take(N4), o_yl = take(N4), o_sf = take(N4);
    size_t o_dtf = take(4 * qn);
    size_t o_in = take(N4), o_perm = take(N4);
    size_t o_md = take(sizeof(emp_model_desc) * (size_t)S);
    size_t o_off = take(8 * (size_t)(S + 1)), o_t0 = take(8 * (size_t)S), o_ord = take(4 * (size_t)S);
    cudaError_t e = cudaMalloc(&h->dbuf, bytes);
    if (e != cudaSuccess) {
        delete h;
        return fail(EMP_E_CUDA, "cudaMalloc(%zu) failed: %s", bytes, cudaGetErrorString(e));
    }
    char* b = (char*)h->dbuf;
    struct Cp { size_t off; const void* src; size_t n; } cps[] = {
        {o_t, H.t.data(), N8}, {o_y, H.y.data(), N8}, {o_s2, H.s2.data(), N8}, {o_dt, hdt.data(), 8 * qn},
        {o_th, H.t_hi.data(), N4}, {o_tl, H.t_lo.data(), N4}, {o_yf, H.y32.data(), N4},
        {o_yl, H.y_lo.data(), N4},
        {o_sf, H.s2_32.data(), N4}, {o_dtf, dtf.data(), 4 * qn}, {o_in, H.inst.data(), N4},
        {o_perm, H.orig.data(), N4}, {o_md, models, sizeof(emp_model_desc) * (size_t)S},
        {o_off, off.data(), 8 * (size_t)(S + 1)}, {o_t0, t0.data(), 8 * (size_t)S},
        {o_ord, sorder.data(), 4 * (size_t)S}};
    for (auto& c : cps) {
        e = cudaMemcpy(b + c.off, c.src, c.n, cudaMemcpyHostToDevice);
        if (e != cudaSuccess) {
            cudaFree(h->dbuf);
            delete h;
            return fail(EMP_E_CUDA, "cudaMemcpy failed: %s", cudaGetErrorString(e));
        }
    }
    h->md_dev = (emp_model_desc*)(b + o_md);
    h->dev2orig = (int*)(b + o_perm);
    if (S > 1) {
        h->sys_off = (const int64_t*)(b + o_off);
        h->sys_t0 = (const double*)(b + o_t0);
        h->sys_order = (const int*)(b + o_ord);
    }
    h->dd.n = n;
    h->dd.q = q;
    h->dd.t0 = t0[0];
    h->dd.t = (const double*)(b + o_t);
    h->dd.y = (const double*)(b + o_y);
    h->dd.s2 = (const double*)(b + o_s2);
    h->dd.dt = (const double*)(b + o_dt);
    h->dd.t_hi = (const float*)(b + o_th);
    h->dd.t_lo = (const float*)(b + o_tl);
    h->dd.y32 = (const float*)(b + o_yf);
    h->dd.y_lo = (const float*)(b + o_yl);
    h->dd.s2_32 = (const float*)(b + o_sf);
    h->dd.dt32 = (const float*)(b + o_dtf);
    h->dd.inst = (const int*)(b + o_in);
    *out = h;
    return EMP_OK;
}

}  // namespace

extern "C" {

int emp_create(const emp_model_desc* model, const emp_dataset_desc* data, emp_handle** out) {
    if (out) *out = nullptr;
    if (data && data->n_systems != 1)
        return fail(EMP_E_UNSUPPORTED, "n_systems=%d: this entry takes one system (emp_create_batch "
                    "takes many)", data->n_systems);
    return create_impl(model, 1, data, out);
}

int emp_create_batch(const emp_model_desc* models, const emp_dataset_desc* data, emp_handle** out) {
    if (out) *out = nullptr;
    if (!data) return fail(EMP_E_INVALID, "dataset descriptor is NULL");
    if (data->n_systems < 1 || data->n_systems > (1 << 20))
        return fail(EMP_E_SIZE, "n_systems=%d outside [1, 2^20]", data->n_systems);
    return create_impl(models, data->n_systems, data, out);
}

int emp_num_systems(emp_handle* h) {
    if (!h) return fail(EMP_E_INVALID, "handle is NULL");
    return h->n_sys;
}

int emp_destroy(emp_handle* h) {
    if (!h) return EMP_OK;
    h->gc.reset();
    h->gch.reset();
    if (h->own) cudaStreamDestroy(h->own);
    if (h->aux) cudaStreamDestroy(h->aux);
    if (h->dbuf) cudaFree(h->dbuf);
    if (h->gp_buf) cudaFree(h->gp_buf);
    if (h->grad_buf) cudaFree(h->grad_buf);
    if (h->am_buf) cudaFree(h->am_buf);
    if (h->am_rows_buf) cudaFree(h->am_rows_buf);
    delete h;
    return EMP_OK;
}

int emp_set_launch(emp_handle* h, int precision, int lanes_per_walker, int tile_epochs) {
    if (!h) return fail(EMP_E_INVALID, "handle is NULL");
    if (precision == EMP_LAUNCH_GRAD) {
        if (lanes_per_walker != 0 && lanes_per_walker != 32)
            return fail(EMP_E_INVALID, "the adjoint kernel runs 32 lanes per walker, not %d", lanes_per_walker);
        if (tile_epochs != 0 && (tile_epochs < 32 || tile_epochs > 4096 || tile_epochs % 32))
            return fail(EMP_E_INVALID, "adjoint tile %d: a multiple of 32 in [32, 4096]", tile_epochs);
        h->grad_tile = tile_epochs;
        return EMP_OK;
    }
    if (precision != EMP_PREC_FP64 && precision != EMP_PREC_MIXED)
        return fail(EMP_E_INVALID, "precision %d unknown", precision);
    if (lanes_per_walker != 0 && lanes_index(lanes_per_walker) < 0)
        return fail(EMP_E_INVALID, "lanes per walker %d not in {8,16,32,64,128,256}", lanes_per_walker);
    if (tile_epochs < 0 || tile_epochs > 16384)
        return fail(EMP_E_INVALID, "tile %d outside [0, 16384]", tile_epochs);
    h->L[precision] = lanes_per_walker;
    h->tile[precision] = tile_epochs;
    h->gc.reset();
    h->gch.reset();
    return EMP_OK;
}

int emp_get_launch(emp_handle* h, int precision, int* lanes_per_walker, int* tile_epochs) {
    if (!h || !lanes_per_walker || !tile_epochs) return fail(EMP_E_INVALID, "NULL argument");
    if (precision != EMP_PREC_FP64 && precision != EMP_PREC_MIXED)
        return fail(EMP_E_INVALID, "precision %d unknown", precision);
    int L = handle_L(h, precision);
    int NT = L > 128 ? L : 128;
    Smem lay;
    *lanes_per_walker = L;
    *tile_epochs = pick_tile(h, precision, L, NT / L, lay);
    return EMP_OK;
}

int emp_logpost(emp_handle* h, const double* theta, int B, const int32_t* system_of,
                const double* beta, double* logl, double* logprior, double* logp, int precision,
                void* stream) {
    if (!h) return fail(EMP_E_INVALID, "handle is NULL");
    if (B < 0) return fail(EMP_E_INVALID, "B=%d < 0", B);
    if (B == 0) return EMP_OK;
    if (!theta || !logl || !logprior) return fail(EMP_E_INVALID, "theta/logl/logprior NULL");
    if (system_of != nullptr)
        return fail(EMP_E_UNSUPPORTED, "system_of must be NULL (a batch handle takes B rows per system)");
    if ((int64_t)B * h->n_sys > 0x7fffffff) return fail(EMP_E_SIZE, "B*systems exceeds 2^31-1");
    KArgs a{};
    a.mode = kModeLogpost;
    a.nwalk = B;
    a.theta = theta;
    a.beta = beta;
    a.logl = logl;
    a.logprior = logprior;
    a.logp = logp;
    int rc = gp_reserve(h, B);
    if (rc) return rc;
    return launch_eval(h, precision, a, (cudaStream_t)stream);
}

int emp_set_astrometry(emp_handle* h, const emp_am_desc* am) {
    if (!h) return fail(EMP_E_INVALID, "handle is NULL");
    if (!am) return fail(EMP_E_INVALID, "astrometry descriptor is NULL");
    if (!h->md.am_on) return fail(EMP_E_INVALID, "the handle's model has no astrometry");
    // one descriptor per system (a batch handle's systems in order); every
    // array is checked before anything reaches the device
    const int S = h->n_sys;
    std::vector<size_t> offs((size_t)S * 7);
    size_t total = 0;
    for (int sy = 0; sy < S; ++sy) {
        const emp_am_desc* a = am + sy;
        if (a->n_hipp < 1 || a->n_gost < 5)
            return fail(EMP_E_INVALID, "system %d: astrometry needs Hipparcos abscissae and at least 5 Gaia epochs",
                        sy);
        if (!a->catalogs || !a->inv_cov || !a->log_det_cov || !a->astro_gost || !a->hipp || !a->gost || !a->gsv)
            return fail(EMP_E_INVALID, "system %d: an astrometry array is NULL", sy);
        const size_t nh = (size_t)a->n_hipp, ng = (size_t)a->n_gost;
        const size_t counts[7] = {21, 75, 3, 10, 7 * nh, 4 * ng, 10 * ng};
        const double* srcs[7] = {a->catalogs, a->inv_cov, a->log_det_cov, a->astro_gost, a->hipp, a->gost, a->gsv};
        for (int k = 0; k < 7; ++k) {
            offs[(size_t)sy * 7 + k] = total;
            total += (8 * counts[k] + 255) & ~(size_t)255;
            for (size_t i = 0; i < counts[k]; ++i)
                if (!isfinite(srcs[k][i]))
                    return fail(EMP_E_INVALID, "system %d: astrometry array %d holds a non-finite value", sy, k);
        }
    }
    const size_t o_dev = total;
    if (S > 1) total += sizeof(AmDev) * (size_t)S;
    if (h->am_buf) {
        cudaFree(h->am_buf);
        h->am_buf = nullptr;
        h->am_sys = nullptr;
        h->am_set = false;
    }
    CUDA_TRY(cudaMalloc(&h->am_buf, total));
    char* b = (char*)h->am_buf;
    std::vector<AmDev> devs((size_t)S);
    for (int sy = 0; sy < S; ++sy) {
        const emp_am_desc* a = am + sy;
        const size_t nh = (size_t)a->n_hipp, ng = (size_t)a->n_gost;
        const size_t counts[7] = {21, 75, 3, 10, 7 * nh, 4 * ng, 10 * ng};
        const double* srcs[7] = {a->catalogs, a->inv_cov, a->log_det_cov, a->astro_gost, a->hipp, a->gost, a->gsv};
        const size_t* o = &offs[(size_t)sy * 7];
        for (int k = 0; k < 7; ++k) CUDA_TRY(cudaMemcpy(b + o[k], srcs[k], 8 * counts[k], cudaMemcpyHostToDevice));
        AmDev& d = devs[(size_t)sy];
        d.n_hipp = a->n_hipp;
        d.n_gost = a->n_gost;
        d.catalogs = (const double*)(b + o[0]);
        d.inv_cov = (const double*)(b + o[1]);
        d.log_det_cov = (const double*)(b + o[2]);
        d.astro_gost = (const double*)(b + o[3]);
        d.hipp = (const double*)(b + o[4]);
        d.gost = (const double*)(b + o[5]);
        d.gsv = (const double*)(b + o[6]);
        d.common_t = a->common_t;
    }
    if (S > 1) {
        CUDA_TRY(cudaMemcpy(b + o_dev, devs.data(), sizeof(AmDev) * (size_t)S, cudaMemcpyHostToDevice));
        h->am_sys = (const AmDev*)(b + o_dev);
    }
    h->am = devs[0];
    h->am_set = true;
    h->gc.reset();
    h->gch.reset();
    return EMP_OK;
}

int emp_model_eval(emp_handle* h, const double* theta, int B, double* model, double* err2,
                   void* stream) {
    if (!h) return fail(EMP_E_INVALID, "handle is NULL");
    if (B < 0) return fail(EMP_E_INVALID, "B=%d < 0", B);
    if (B == 0) return EMP_OK;
    if (B > 65535) return fail(EMP_E_SIZE, "B=%d > 65535", B);
    if (!theta || !model || !err2) return fail(EMP_E_INVALID, "NULL argument");
    if (h->n_sys > 1) return fail(EMP_E_UNSUPPORTED, "model evaluation takes a one-system handle");
    cudaStream_t s = (cudaStream_t)stream;
    const emp_model_desc& m = h->md;
    size_t sm = 8 * ((size_t)m.n_full + 8 * std::max(m.n_planets, 1) + 2 * m.n_ins + std::max(m.acc_order, 1));
    dim3 grid((unsigned)std::min(64, (h->n + 255) / 256), (unsigned)B);
    k_model_mean<<<grid, 256, sm, s>>>(h->md_dev, h->dd, h->dev2orig, theta, model, err2);
    g_launches.fetch_add(1);
    CUDA_TRY(cudaGetLastError());
    if (h->q > 0) {
        k_model_ma<<<(B + 127) / 128, 128, 0, s>>>(h->md_dev, h->dd, h->dev2orig, theta, B, model);
        g_launches.fetch_add(1);
        CUDA_TRY(cudaGetLastError());
    }
    return EMP_OK;
}

int emp_gp_logl(emp_handle* h, const double* theta, int B, const double* resid, const double* err2,
                double* logl, int precision, void* stream) {
    if (!h) return fail(EMP_E_INVALID, "handle is NULL");
    if (precision != EMP_PREC_FP64 && precision != EMP_PREC_MIXED)
        return fail(EMP_E_INVALID, "precision %d unknown", precision);
    if (h->gp_M == 0) return fail(EMP_E_UNSUPPORTED, "the handle's model has no GP");
    if (h->n_sys > 1) return fail(EMP_E_UNSUPPORTED, "emp_gp_logl takes a one-system handle");
    if (B < 0) return fail(EMP_E_INVALID, "B=%d < 0", B);
    if (B == 0) return EMP_OK;
    if (!theta || !resid || !err2 || !logl) return fail(EMP_E_INVALID, "a NULL argument");
    int rc = gp_reserve(h, B);
    if (rc) return rc;
    KArgs a{};
    a.md = h->md_dev;
    a.d = h->dd;
    a.mode = kModeGPOnly;
    a.nwalk = B;
    a.theta = theta;
    a.logl = logl;
    a.dstride = h->lay[1];
    gp_args(h, a);
    cudaStream_t s = (cudaStream_t)stream;
    if (precision == EMP_PREC_FP64) {
        a.gp_r = const_cast<double*>(resid);
        a.gp_e = const_cast<double*>(err2);
    } else {
        // float-float rows in the handle's residual buffers
        const size_t count = (size_t)h->n * B;
        const int grid = (int)std::min<size_t>((count + 255) / 256, (size_t)std::max(1, h->sms) * 8);
        k_gp_cvt<<<grid, 256, 0, s>>>(resid, err2, reinterpret_cast<float2*>(h->gp_r),
                                      reinterpret_cast<float2*>(h->gp_e), count);
        g_launches.fetch_add(1);
        CUDA_TRY(cudaGetLastError());
    }
    return launch_gp(h, a, s, precision);
}

int emp_logpost_grad(emp_handle* h, const double* theta, int B, double* logl, double* logprior,
                     double* grad_logl, double* grad_logprior, void* stream) {
    if (!h) return fail(EMP_E_INVALID, "handle is NULL");
    if (B < 0) return fail(EMP_E_INVALID, "B=%d < 0", B);
    if (B == 0) return EMP_OK;
    if (!theta || !logl || !logprior || !grad_logl || !grad_logprior)
        return fail(EMP_E_INVALID, "a NULL argument");
    if (h->n_sys > 1) return fail(EMP_E_UNSUPPORTED, "the gradient takes a one-system handle");
    if (h->gp_M > 0) return fail(EMP_E_UNSUPPORTED, "gradient: GP likelihoods are not built");
    if (h->md.am_on) return fail(EMP_E_UNSUPPORTED, "gradient: the astrometric likelihood is not built");
    const emp_model_desc& m = h->md;
    if (m.n_ins > kGradMaxIns)
        return fail(EMP_E_UNSUPPORTED, "gradient: %d instruments (at most %d)", m.n_ins, kGradMaxIns);
    if (h->q > 3) return fail(EMP_E_UNSUPPORTED, "gradient: MA order %d (at most 3)", h->q);
    constexpr int L = 32, NT = 128, G = NT / L;
    const int n = h->n;
    // the epoch tile: the caller's, else the series rounded up to 32 lanes,
    // halved while the CTA would leave fewer than four CTAs per SM
    int tile = h->grad_tile;
    if (tile == 0) {
        tile = std::min(1024, ((n + L - 1) / L) * L);
        GSmem l2;
        for (;;) {
            l2.build(h->q, L, G, tile, m.n_full, m.n_free, m.n_planets, m.n_ins, m.acc_order);
            if (l2.total * 4 <= 224 * 1024 || tile <= 256) break;
            tile = std::max(256, tile / 2);
        }
    }
    GSmem lay;
    lay.build(h->q, L, G, tile, m.n_full, m.n_free, m.n_planets, m.n_ins, m.acc_order);
    if (lay.total > 227 * 1024)
        return fail(EMP_E_SIZE, "gradient: tile of %d epochs needs %d B of shared memory", tile, lay.total);
    const int ntiles = (n + tile - 1) / tile;
    const int64_t stride = (int64_t)ntiles * tile;
    float* resid = nullptr;
    if (h->q > 0 && ntiles > 1) {
        // residuals between the forward and backward passes: B rows of the
        // tiled series, allocated on first need (outside any capture)
        const size_t need = (size_t)B * (size_t)stride * sizeof(float);
        if (need > h->grad_bytes) {
            if (h->grad_buf) CUDA_TRY(cudaFree(h->grad_buf));
            h->grad_buf = nullptr;
            h->grad_bytes = 0;
            CUDA_TRY(cudaMalloc(&h->grad_buf, need));
            h->grad_bytes = need;
        }
        resid = static_cast<float*>(h->grad_buf);
    }
    GFn fn = get_kernel_grad(h->q, 0);
    if (!fn) return fail(EMP_E_UNSUPPORTED, "no gradient kernel for q=%d", h->q);
    if (!h->grad_attr[h->q]) {
        CUDA_TRY(cudaFuncSetAttribute((const void*)fn, cudaFuncAttributeMaxDynamicSharedMemorySize, 227 * 1024));
        h->grad_attr[h->q] = true;
    }
    GArgs a{};
    a.md = h->md_dev;
    a.d = h->dd;
    a.nwalk = B;
    a.tile = tile;
    a.theta = theta;
    a.logl = logl;
    a.logprior = logprior;
    a.grad_logl = grad_logl;
    a.grad_logprior = grad_logprior;
    a.resid = resid;
    a.resid_stride = stride;
    fn<<<(B + G - 1) / G, NT, lay.total, (cudaStream_t)stream>>>(a);
    g_launches.fetch_add(1);
    CUDA_TRY(cudaGetLastError());
    return EMP_OK;
}

int64_t emp_pt_work_bytes(int ntemps, int nwalkers, int ndim) {
    (void)ndim;
    if (ntemps < 1 || nwalkers < 1) return 0;
    return (int64_t)work_bytes(ntemps, nwalkers);
}

int emp_pt_evaluate(emp_handle* h, const emp_pt_state* st, void* stream) {
    if (!h) return fail(EMP_E_INVALID, "handle is NULL");
    int rc = check_state(h, st);
    if (rc) return rc;
    KArgs a{};
    a.mode = kModeSlots;
    a.nwalk = st->ntemps * st->nwalkers;
    a.T = st->ntemps;
    a.W = st->nwalkers;
    a.st_theta = st->theta;
    a.st_logl = st->logl;
    a.st_logprior = st->logprior;
    if ((rc = gp_reserve(h, (int64_t)st->ntemps * st->nwalkers))) return rc;
    if ((rc = am_reserve(h, (int64_t)st->ntemps * st->nwalkers))) return rc;
    return launch_eval(h, st->precision, a, (cudaStream_t)stream);
}

int emp_pt_sweep(emp_handle* h, const emp_pt_state* st, const emp_pt_record* rec, void* stream) {
    if (!h) return fail(EMP_E_INVALID, "handle is NULL");
    int rc = check_state(h, st);
    if (rc) return rc;
    if ((rc = gp_reserve(h, (int64_t)st->ntemps * st->nwalkers))) return rc;
    if ((rc = am_reserve(h, (int64_t)st->ntemps * st->nwalkers))) return rc;
    return enqueue_sweep(h, st, rec, (cudaStream_t)stream, nullptr);
}

}  // extern "C"

// ---------------------------------------------------------------------------
// Sweep without any allocation by the caller or the library.
//
// Some callers cannot call cudaMalloc at all: host programs whose device
// memory is one fixed arena handed out by their own allocator (a second
// allocator would fragment or overcommit it), and processes that forbid any
// allocation once they are running (real-time loops, allocation-audited
// services).  emp_pt_sweep_static serves them: the sweep's workspace (the
// swap log, the per-sweep rows, the ladder of the running sweep) lives in
// the file-scope array below instead of a caller buffer.
//
// The array holds one PT state of up to kStaticMaxWalkers = ntemps*nwalkers
// walkers (about 260 KB); every GPU that loads this library keeps it until
// the process exits.  All calls share it and it keeps the last call's
// contents, so each call first clears the part that must start at zero;
// calls that overlap on the GPU (other streams, other threads) race on it.
// The first call on each device looks the array's device address up
// (cudaGetSymbolAddress, with that device current) and sets the kernels'
// attributes; that first call should come before any stream capture.
// ---------------------------------------------------------------------------
static constexpr int kStaticMaxWalkers = 32768;
static constexpr size_t kStaticHeaderBytes = work_bytes(0, 0);
static constexpr size_t kStaticWorkBytes = (work_bytes(1, kStaticMaxWalkers) + 255) & ~(size_t)255;
static_assert(kStaticHeaderBytes == kWorkHeaderBytes, "static workspace header out of step with Work");
static __device__ __align__(256) unsigned char g_static_work[kStaticWorkBytes];

static std::mutex g_static_mu;
static void* g_static_ptr[64] = {};

// device address of g_static_work on the current device; looked up once per
// device (the host-side name of the array is not a device address)
static int static_work_address(void** out) {
    int dev = 0;
    CUDA_TRY(cudaGetDevice(&dev));
    if (dev < 0 || dev >= 64) return fail(EMP_E_INVALID, "device %d out of range", dev);
    std::lock_guard<std::mutex> lk(g_static_mu);
    if (!g_static_ptr[dev]) {
        void* p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_static_work);
        if (e != cudaSuccess || p == nullptr)
            return fail(EMP_E_CUDA, "cudaGetSymbolAddress(static workspace): %s", cudaGetErrorString(e));
        g_static_ptr[dev] = p;
    }
    *out = g_static_ptr[dev];
    return EMP_OK;
}

extern "C" int emp_pt_sweep_static(emp_handle* h, const emp_pt_state* st, const emp_pt_record* rec,
                                   void* stream) {
    if (!h) return fail(EMP_E_INVALID, "handle is NULL");
    if (!st) return fail(EMP_E_INVALID, "state is NULL");
    const int64_t walkers = (int64_t)st->ntemps * st->nwalkers;
    if (walkers > kStaticMaxWalkers)
        return fail(EMP_E_SIZE, "ntemps*nwalkers=%lld exceeds the static workspace limit of %d walkers",
                    (long long)walkers, kStaticMaxWalkers);
    void* ws = nullptr;
    int rc = static_work_address(&ws);
    if (rc) return rc;
    emp_pt_state local = *st;
    local.work = ws;
    local.work_bytes = (int64_t)kStaticWorkBytes;
    if ((rc = check_state(h, &local))) return rc;
    if (h->md.am_on && h->am_rows < walkers)
        return fail(EMP_E_UNSUPPORTED, "a model with astrometry needs its row workspace (emp_pt_evaluate or "
                    "emp_pt_sweep allocates it) before the allocation-free sweep");
    if (h->gp_M > 0 && h->gp_rows < walkers)
        return fail(EMP_E_UNSUPPORTED, "a GP model needs its row workspace (emp_pt_evaluate or emp_pt_sweep "
                    "allocates it) before the allocation-free sweep");
    if ((rc = prepare_sweep(h, local.precision))) return rc;
    cudaStream_t s = (cudaStream_t)stream;
    CUDA_TRY(cudaMemsetAsync(ws, 0, kStaticHeaderBytes, s));
    return enqueue_sweep(h, &local, rec, s, nullptr);
}

namespace {

// Capture one sweep into gc (replacing what it held): with `host` non-null
// the packed walker state is copied in from `host` before the sweep and back
// after it, inside the graph.  Kernel attributes and the persistent grid are
// set up before the capture (it forbids cudaFuncSetAttribute side effects on
// some drivers).
int capture_sweep(emp_handle* h, GraphCache& gc, const emp_pt_state* st, const emp_pt_record* rec,
                  cudaStream_t ls, void* host, size_t host_bytes) {
    int rc;
    emp_pt_record rcopy{};
    const bool has_rec = rec != nullptr;
    if (has_rec) rcopy = *rec;
    gc.reset();
    if ((rc = prepare_sweep(h, st->precision))) return rc;
    HostCopy hc{};
    if (host) {
        if (!h->aux) CUDA_TRY(cudaStreamCreateWithFlags(&h->aux, cudaStreamNonBlocking));
        hc.host = host;
        hc.bytes = host_bytes;
        hc.aux = h->aux;
        CUDA_TRY(cudaEventCreateWithFlags(&hc.ev[0], cudaEventDisableTiming));
        cudaError_t e1 = cudaEventCreateWithFlags(&hc.ev[1], cudaEventDisableTiming);
        if (e1 != cudaSuccess) {
            cudaEventDestroy(hc.ev[0]);
            return fail(EMP_E_CUDA, "cudaEventCreate: %s", cudaGetErrorString(e1));
        }
    }
    auto drop_events = [&]() {
        if (host) { cudaEventDestroy(hc.ev[0]); cudaEventDestroy(hc.ev[1]); }
    };
    {
        cudaError_t e0 = cudaStreamBeginCapture(ls, cudaStreamCaptureModeThreadLocal);
        if (e0 != cudaSuccess) {
            drop_events();
            return fail(EMP_E_CUDA, "cudaStreamBeginCapture: %s", cudaGetErrorString(e0));
        }
    }
    int nk = 0;
    int64_t before = g_launches.load();
    rc = EMP_OK;
    if (host) {
        cudaError_t e = cudaMemcpyAsync(st->theta, host, host_bytes, cudaMemcpyHostToDevice, ls);
        if (e != cudaSuccess) rc = fail(EMP_E_CUDA, "state copy in: %s", cudaGetErrorString(e));
    }
    if (!rc) rc = enqueue_sweep(h, st, has_rec ? &rcopy : nullptr, ls, &nk, host ? &hc : nullptr);
    g_launches.store(before);   // captured, not launched
    cudaGraph_t graph = nullptr;
    cudaError_t e = cudaStreamEndCapture(ls, &graph);
    drop_events();
    if (rc) {
        if (graph) cudaGraphDestroy(graph);
        return rc;
    }
    if (e != cudaSuccess) return fail(EMP_E_CUDA, "cudaStreamEndCapture: %s", cudaGetErrorString(e));
    cudaGraphExec_t exec = nullptr;
    e = cudaGraphInstantiate(&exec, graph, 0);
    if (e != cudaSuccess) {
        cudaGraphDestroy(graph);
        return fail(EMP_E_CUDA, "cudaGraphInstantiate: %s", cudaGetErrorString(e));
    }
    gc.graph = graph;
    gc.exec = exec;
    gc.st = *st;
    gc.rec = rcopy;
    gc.has_rec = has_rec;
    gc.stream = ls;
    gc.host = host;
    gc.kernels_per_launch = nk;
    gc.valid = true;
    return EMP_OK;
}

bool graph_matches(const GraphCache& gc, const emp_pt_state* st, const emp_pt_record* rec, cudaStream_t ls,
                   void* host) {
    const bool has_rec = rec != nullptr;
    return gc.valid && gc.stream == ls && gc.host == host && same_state(gc.st, *st) && gc.has_rec == has_rec &&
           (!has_rec || same_rec(gc.rec, *rec));
}

// launch the captured graph `times` times on ls, ordered after and before the
// caller's stream s
int launch_graph(GraphCache& gc, cudaStream_t s, cudaStream_t ls, int times) {
    cudaEvent_t ev = nullptr;
    if (ls != s) {
        CUDA_TRY(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming));
        CUDA_TRY(cudaEventRecord(ev, s));
        CUDA_TRY(cudaStreamWaitEvent(ls, ev, 0));
    }
    for (int i = 0; i < times; ++i) {
        cudaError_t e = cudaGraphLaunch(gc.exec, ls);
        if (e != cudaSuccess) {
            if (ev) cudaEventDestroy(ev);
            return fail(EMP_E_CUDA, "cudaGraphLaunch: %s", cudaGetErrorString(e));
        }
        g_launches.fetch_add(gc.kernels_per_launch);
    }
    if (ls != s) {
        CUDA_TRY(cudaEventRecord(ev, ls));
        CUDA_TRY(cudaStreamWaitEvent(s, ev, 0));
        cudaEventDestroy(ev);
    }
    return EMP_OK;
}

// graphs are captured and launched on a non-legacy stream
int launch_stream(emp_handle* h, cudaStream_t s, cudaStream_t* ls) {
    *ls = s;
    if (s == nullptr || s == cudaStreamLegacy) {
        if (!h->own) CUDA_TRY(cudaStreamCreateWithFlags(&h->own, cudaStreamNonBlocking));
        *ls = h->own;
    }
    return EMP_OK;
}

}  // namespace

extern "C" {

int emp_pt_run(emp_handle* h, const emp_pt_state* st, const emp_pt_record* rec, int nsweeps,
               int use_graph, void* stream) {
    if (!h) return fail(EMP_E_INVALID, "handle is NULL");
    int rc = check_state(h, st);
    if (rc) return rc;
    if (nsweeps < 0) return fail(EMP_E_INVALID, "nsweeps=%d < 0", nsweeps);
    if (nsweeps == 0) return EMP_OK;
    if ((rc = gp_reserve(h, (int64_t)st->ntemps * st->nwalkers))) return rc;
    if ((rc = am_reserve(h, (int64_t)st->ntemps * st->nwalkers))) return rc;
    cudaStream_t s = (cudaStream_t)stream;
    if (!use_graph) {
        for (int i = 0; i < nsweeps; ++i)
            if ((rc = enqueue_sweep(h, st, rec, s, nullptr))) return rc;
        return EMP_OK;
    }
    cudaStream_t ls;
    if ((rc = launch_stream(h, s, &ls))) return rc;
    if (!graph_matches(h->gc, st, rec, ls, nullptr))
        if ((rc = capture_sweep(h, h->gc, st, rec, ls, nullptr, 0))) return rc;
    return launch_graph(h->gc, s, ls, nsweeps);
}

int emp_pt_run_host(emp_handle* h, const emp_pt_state* st, const emp_pt_record* rec, void* host_state,
                    void* stream) {
    if (!h) return fail(EMP_E_INVALID, "handle is NULL");
    int rc = check_state(h, st);
    if (rc) return rc;
    if (!host_state) return fail(EMP_E_INVALID, "host state is NULL");
    if (h->n_sys > 1) return fail(EMP_E_UNSUPPORTED, "the host-state sweep takes a one-system handle");
    const size_t tw = (size_t)st->ntemps * st->nwalkers;
    if (st->logl != st->theta + tw * st->ndim || st->logprior != st->logl + tw)
        return fail(EMP_E_INVALID, "state buffers not packed (theta rows, then logl, then logprior)");
    cudaPointerAttributes pa{};
    CUDA_TRY(cudaPointerGetAttributes(&pa, host_state));
    if (pa.type != cudaMemoryTypeHost) return fail(EMP_E_INVALID, "host state is not page-locked host memory");
    if ((rc = gp_reserve(h, (int64_t)tw))) return rc;
    if ((rc = am_reserve(h, (int64_t)tw))) return rc;
    cudaStream_t s = (cudaStream_t)stream, ls;
    if ((rc = launch_stream(h, s, &ls))) return rc;
    if (!graph_matches(h->gch, st, rec, ls, host_state))
        if ((rc = capture_sweep(h, h->gch, st, rec, ls, host_state, tw * (st->ndim + 2) * sizeof(double))))
            return rc;
    return launch_graph(h->gch, s, ls, 1);
}

int emp_probe_peaks(double* fp32_flops, double* fp64_flops, void* stream) {
    if (!fp32_flops || !fp64_flops) return fail(EMP_E_INVALID, "NULL output");
    int dev = 0, sms = 0;
    CUDA_TRY(cudaGetDevice(&dev));
    CUDA_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    cudaStream_t s = (cudaStream_t)stream;
    void* out = nullptr;
    CUDA_TRY(cudaMalloc(&out, 8 * 4096));
    cudaEvent_t e0, e1;
    CUDA_TRY(cudaEventCreate(&e0));
    CUDA_TRY(cudaEventCreate(&e1));
    const int blocks = sms * 8, threads = 256;
    double res[2] = {0, 0};
    for (int which = 0; which < 2; ++which) {
        int iters = which == 0 ? 4096 : 64;
        float best = 1e30f;
        for (int rep = 0; rep < 4; ++rep) {
            cudaEventRecord(e0, s);
            if (which == 0) k_fma_probe<float><<<blocks, threads, 0, s>>>((float*)out, iters, 1.0f);
            else k_fma_probe<double><<<blocks, threads, 0, s>>>((double*)out, iters, 1.0);
            cudaEventRecord(e1, s);
            g_launches.fetch_add(1);
            cudaError_t e = cudaEventSynchronize(e1);
            if (e != cudaSuccess) {
                cudaFree(out);
                return fail(EMP_E_CUDA, "probe: %s", cudaGetErrorString(e));
            }
            float ms = 0.f;
            cudaEventElapsedTime(&ms, e0, e1);
            if (rep > 0) best = std::min(best, ms);
        }
        double flops = 2.0 * 8 * 16 * (double)iters * blocks * threads;
        res[which] = flops / (best * 1e-3);
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFree(out);
    *fp32_flops = res[0];
    *fp64_flops = res[1];
    return EMP_OK;
}

}  // extern "C"
