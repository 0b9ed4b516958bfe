// sphmp_api.cu — the C ABI (include/sphmp.h, include/sphmp_legacy.h): context
// lifetime, host transfers, per-pass entry points, the graph-captured step and
// the reference's own entry-point names over a default context.
#include <cuda_runtime.h>
#include <math.h>
#include <stdarg.h>
#include <stdio.h>
#include <string.h>

#include <algorithm>
#include <mutex>
#include <string>
#include <utility>
#include <vector>

#include "sphmp.h"
#include "sphmp_emit.h"
#include "sphmp_internal.h"
#include "sphmp_learned.h"
#include "sphmp_legacy.h"

using namespace sphmp;

struct sphmp_ctx {
    sphmp_params prm;
    int cap = 0;         // particle capacity
    int gcap = 0;        // grid cells allocated
    int corder_res[3] = {0, 0, 0};  // grid the Z-order cell permutation (B.corder) was built for
    int n = 0;           // active slots
    int cur[kNumFloat4Fields] = {0, 0, 0, 0, 0};
    bool alpha_advanced = false;  // alpha4[cur] = advanced fractions, alpha4[cur^1] = start of step
    bool grid_valid = false;      // cell starts built for the current slot order
    bool nbr_valid = false;       // neighbour list built by the density pass for the current positions
    bool oct_built = false;       // the last grid list also built the next internal order (osrc)
    bool oct_valid = false;       // the internal order is octant-grouped for the current cell list
    bool pos_sorted = false;      // positions unchanged since the cell list was built from them
    int hash_n = -1;              // particle count the cell keys were computed for (-1: none)
    int list_mode = 0;            // kind of list the last density pass wrote (DevParams::list_mode)
    int device = 0;
    cudaStream_t own_stream = nullptr;
    cudaStream_t stream = nullptr;
    DevBuffers B{};
    void* stage = nullptr;  // device staging: reference records / field arrays
    size_t stage_bytes = 0;
    cudaGraphExec_t graph = nullptr;
    int graph_n = -1;
    int graph_schedule = -1;
    int graph_cur[kNumFloat4Fields] = {0, 0, 0, 0, 0};  // the buffer selectors the graph was captured with
    // asynchronous display downloads: two device staging buffers, copied to the
    // host on a separate stream while the context stream runs on
    cudaStream_t copy_stream = nullptr;
    sphmp_display_pack* dl_stage[2] = {nullptr, nullptr};
    cudaEvent_t dl_packed[2] = {nullptr, nullptr};
    cudaEvent_t dl_done[2] = {nullptr, nullptr};
    int dl_next = 0;
    // device-side emission: while `emit_on`, every step starts with the emitter
    // kernel, the kernels run over the capacity and bound themselves by the device
    // count, and `n` is re-read from the device after steps (`n_stale`)
    bool emit_on = false;
    bool n_stale = false;
    DevEmitter emitter{};
    // learned large step (allocated by the first corrected step): per row of the
    // internal order, the features, bornid (-1: no features), network outputs
    // and applied corrections of the last corrected step
    float* lfeat = nullptr;
    int32_t* lids = nullptr;
    float* ly = nullptr;
    float* lcorr = nullptr;
    int lrows = 0;
    void* xstage = nullptr;  // sphmp_copy_state: fractions and (g - a) of the source
    // set by the rollout right after a sort and density pass of its own with no
    // other call since; the next eager large step skips its sort and density
    // pass, which would reproduce them bit for bit
    bool sorted_dens_fresh = false;
    int32_t* cmap = nullptr; // sphmp_compare_states: bornid -> index
    int cmap_size = 0;
    double* cred = nullptr;  // sphmp_compare_states: 6 sums
};

namespace {

thread_local std::string g_err;

sphmp_status fail(sphmp_status st, const char* fmt, ...) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    g_err = buf;
    return st;
}

sphmp_status cuda_fail(cudaError_t e, const char* what) {
    return fail(SPHMP_ERR_CUDA, "%s: %s", what, cudaGetErrorString(e));
}

#define CK(call)                                                    \
    do {                                                            \
        cudaError_t e_ = (call);                                    \
        if (e_ != cudaSuccess) return cuda_fail(e_, #call);         \
    } while (0)

#define CHECK_LAUNCH(what)                                          \
    do {                                                            \
        cudaError_t e_ = cudaGetLastError();                        \
        if (e_ != cudaSuccess) return cuda_fail(e_, what);          \
    } while (0)

// Z-order (Morton) code of a cell: the bits of gx, gz and gy interleaved, x lowest.
uint64_t morton_code(uint32_t gx, uint32_t gy, uint32_t gz) {
    uint64_t m = 0;
    for (int b = 0; b < 21; b++) {
        m |= (uint64_t)((gx >> b) & 1u) << (3 * b);
        m |= (uint64_t)((gz >> b) & 1u) << (3 * b + 1);
        m |= (uint64_t)((gy >> b) & 1u) << (3 * b + 2);
    }
    return m;
}

sphmp_status validate_params(const sphmp_params* p) {
    if (!p) return fail(SPHMP_ERR_INVALID_ARG, "params is NULL");
    if (p->maxNum <= 0) return fail(SPHMP_ERR_INVALID_ARG, "maxNum must be > 0 (got %d)", p->maxNum);
    if (p->num < 0 || p->num > p->maxNum) return fail(SPHMP_ERR_CAPACITY, "num %d outside [0, maxNum=%d]", p->num, p->maxNum);
    if (p->nphase < 1 || p->nphase > SPHMP_MAX_PHASES)
        return fail(SPHMP_ERR_INVALID_ARG, "nphase must be 1..3 (got %d)", p->nphase);
    if (!(p->smoothradius > 0.f) || !isfinite(p->smoothradius)) return fail(SPHMP_ERR_NOT_FINITE, "smoothradius must be > 0");
    if (!(p->simscale > 0.f) || !isfinite(p->simscale)) return fail(SPHMP_ERR_NOT_FINITE, "simscale must be > 0");
    if (!isfinite(p->dt)) return fail(SPHMP_ERR_NOT_FINITE, "dt not finite");
    for (int a = 0; a < 3; a++) {
        if (p->gridres[a] < 3) return fail(SPHMP_ERR_GRID, "gridres[%d] = %d < 3 (call sphmp_setup_grid)", a, p->gridres[a]);
        if (!isfinite(p->gridmin[a]) || !(p->gridIdfac[a] > 0.f) || !isfinite(p->gridIdfac[a]))
            return fail(SPHMP_ERR_GRID, "grid origin/factor not finite on axis %d", a);
    }
    const long long g = (long long)p->gridres[0] * p->gridres[1] * p->gridres[2];
    if (g != p->gridtotal) return fail(SPHMP_ERR_GRID, "gridtotal %d != product of gridres %lld", p->gridtotal, g);
    if (g > (1ll << 31) - 16) return fail(SPHMP_ERR_GRID, "grid too large (%lld cells)", g);
    if (p->eos != SPHMP_EOS_TAIT && p->eos != SPHMP_EOS_LINEAR) return fail(SPHMP_ERR_INVALID_ARG, "unknown eos %d", p->eos);
    if (p->cell_order != SPHMP_CELL_ORDER_LINEAR && p->cell_order != SPHMP_CELL_ORDER_MORTON)
        return fail(SPHMP_ERR_INVALID_ARG, "unknown cell order %d", p->cell_order);
    if (p->bucket_window != 0 && (p->bucket_window < (int)kBucketWindowMin || p->bucket_window > (int)kBucketWindow))
        return fail(SPHMP_ERR_INVALID_ARG, "bucket_window must be 0 or 8..32 (got %d)", p->bucket_window);
    if (p->heavy_list != 0 && (p->heavy_list < 32 || p->heavy_list > kMaxNbr))
        return fail(SPHMP_ERR_INVALID_ARG, "heavy_list must be 0 or 32..256 (got %d)", p->heavy_list);
    return SPHMP_OK;
}

DevParams dev_params(const sphmp_ctx* c) {
    const sphmp_params& p = c->prm;
    DevParams P;
    memset(&P, 0, sizeof(P));
    P.n = c->emit_on ? c->cap : c->n;
    P.cap = c->cap;
    P.G = p.gridtotal;
    P.rx = p.gridres[0];
    P.ry = p.gridres[1];
    P.rz = p.gridres[2];
    for (int a = 0; a < 3; a++) {
        P.gmin[a] = p.gridmin[a];
        P.fac[a] = p.gridIdfac[a];
        P.srad[a] = (float)((double)p.smoothradius / (double)p.simscale * (double)p.gridIdfac[a] + 1.0e-3);
        P.grav[a] = p.gravity[a];
    }
    P.ss = p.simscale;
    P.h = p.smoothradius;
    P.r2 = p.smoothradius * p.smoothradius;
    P.r2list = P.r2 * (1.0f + 1.0e-5f);
    P.list_mode = c->nbr_valid ? c->list_mode : 0;
    P.narrow = c->pos_sorted ? 1 : 0;
    P.dt = p.dt;
    P.kpoly6 = p.kpoly6;
    P.kspline = p.kspline;
    P.kspikydiff = p.kspikydiff;
    P.bvisc = p.bvisc;
    P.nphase = p.nphase;
    P.multiphase = p.multiphase;
    for (int k = 0; k < 3; k++) {
        P.dens_k[k] = p.densArr[k];
        P.visc_k[k] = p.viscArr[k];
    }
    P.relax = p.mf_relax;
    P.sigma = p.mf_diffusion;
    P.cont = p.mf_cont;
    P.cont1 = p.mf_cont1;
    P.cont2 = p.mf_cont2;
    P.pintstiff = p.mf_pintstiff;
    P.omega = p.mf_omega;
    P.visc_factor = p.mf_visc_factor;
    P.eos = p.eos;
    P.eos_k = p.eos_stiffness;
    P.st_on = p.surface_tension;
    P.st_K = p.surfaceTensionK;
    P.st_C = p.surfaceTensionFluidC;
    for (int k = 0; k < 27; k++) P.neighborid[k] = p.neighborid[k];
    P.morton = p.cell_order == SPHMP_CELL_ORDER_MORTON;
    P.bwin = p.bucket_window > 0 ? p.bucket_window : (int)kBucketWindow;
    P.heavy = p.heavy_list > 0 ? (uint32_t)p.heavy_list : kHeavyList;
    return P;
}

void drop_graph(sphmp_ctx* c) {
    if (c->graph) cudaGraphExecDestroy(c->graph);
    c->graph = nullptr;
    c->graph_n = -1;
    c->graph_schedule = -1;
}

void free_buffers(sphmp_ctx* c) {
    DevBuffers& B = c->B;
    for (int f = 0; f < kNumFloat4Fields; f++)
        for (int b = 0; b < 2; b++) cudaFree(B.f4[f][b]);
    void* ptrs[] = {B.densp, B.accel4, B.drift4, B.velxcor, B.pmod, B.mgcell, B.midsort, B.mgndx, B.mgridoff, B.mgridcnt,
                    B.key, B.octk, B.arank, B.sidx, B.ccount, B.cstart, B.cend, B.corder, B.bsum, B.uchunk, B.big, B.color, B.bornid,
                    B.mass_raw, B.err, B.red, B.vtmp, B.nbr, B.nbr_cnt, B.nmask, B.btab, B.dctr, B.wq, B.wq_n, B.hq, B.hq_n, B.hctr, B.iis_dii, B.iis_dijpj, B.iis_aii, B.iis_rho_adv, B.iis_pl, B.iis_pl1, B.iis_res, B.nrec, B.opos, B.oidx, B.osrc, B.oct_start,
                    B.act, B.act_n, B.nact, B.frame, c->stage};
    for (void* q : ptrs) cudaFree(q);
    memset(&c->B, 0, sizeof(c->B));
    c->stage = nullptr;
}

template <class T>
cudaError_t dalloc(T** p, size_t count) {
    return cudaMalloc((void**)p, sizeof(T) * (count ? count : 1));
}

sphmp_status alloc_buffers(sphmp_ctx* c) {
    const size_t N = (size_t)c->cap;
    const size_t G = (size_t)c->gcap;
    DevBuffers& B = c->B;
    for (int f = 0; f < kNumFloat4Fields; f++)
        for (int b = 0; b < 2; b++) CK(dalloc(&B.f4[f][b], N));
    CK(dalloc(&B.densp, N));
    CK(dalloc(&B.accel4, N));
    CK(dalloc(&B.drift4, 3 * N));
    CK(dalloc(&B.velxcor, N));
    CK(dalloc(&B.pmod, N));
    CK(dalloc(&B.mgcell, N));
    CK(dalloc(&B.midsort, N));
    CK(dalloc(&B.mgndx, N));
    CK(dalloc(&B.mgridoff, G));
    CK(dalloc(&B.mgridcnt, G));
    CK(dalloc(&B.key, N));
    CK(dalloc(&B.octk, N));
    CK(dalloc(&B.arank, N));
    CK(dalloc(&B.sidx, N));
    CK(dalloc(&B.ccount, G + 1));
    CK(dalloc(&B.cstart, G + 2));
    CK(dalloc(&B.cend, G));
    CK(dalloc(&B.corder, G));
    const size_t per = (size_t)kScanBlock * kScanItems;
    CK(dalloc(&B.bsum, (G + per - 1) / per + 1));
    CK(dalloc(&B.uchunk, N / kHashBlock + 2));
    CK(dalloc(&B.big, N / (kWarpSortMax + 1) + 2));
    CK(dalloc(&B.color, N));
    CK(dalloc(&B.bornid, N));
    CK(dalloc(&B.mass_raw, N));
    CK(dalloc(&B.err, 1));
    CK(dalloc(&B.red, 16));
    CK(dalloc(&B.vtmp, N));
    CK(dalloc(&B.nbr, (size_t)kMaxNbr * N));
    CK(dalloc(&B.nbr_cnt, N));
    CK(dalloc(&B.nmask, (size_t)kMaskWords * N));
    CK(dalloc(&B.btab, 8 * G * kTabStride));
    CK(dalloc(&B.dctr, 1));
    CK(dalloc(&B.wq, N / kBucketWindowMin + 16));
    CK(dalloc(&B.wq_n, 1));
    CK(cudaMemset(B.wq_n, 0, sizeof(uint32_t)));
    CK(dalloc(&B.hq, N));
    CK(dalloc(&B.hq_n, 1));
    CK(dalloc(&B.hctr, 2));
    CK(cudaMemset(B.hq_n, 0, sizeof(uint32_t)));
    CK(dalloc(&B.iis_dii, N));
    CK(dalloc(&B.iis_dijpj, N));
    CK(dalloc(&B.iis_aii, N));
    CK(dalloc(&B.iis_rho_adv, N));
    CK(dalloc(&B.iis_pl, N));
    CK(dalloc(&B.iis_pl1, N));
    CK(dalloc(&B.iis_res, N));
    CK(cudaMemset(B.iis_dii, 0, sizeof(float4) * N));
    CK(cudaMemset(B.iis_dijpj, 0, sizeof(float4) * N));
    CK(cudaMemset(B.iis_pl, 0, sizeof(float) * N));
    CK(cudaMemset(B.iis_res, 0, sizeof(float) * N));
    CK(dalloc(&B.nrec, (size_t)kNrecFloat4 * N));
    CK(dalloc(&B.opos, N));
    CK(dalloc(&B.oidx, N));
    CK(dalloc(&B.osrc, N));
    CK(dalloc(&B.oct_start, 8 * G));
    CK(dalloc(&B.act, G));
    CK(dalloc(&B.act_n, 1));
    CK(cudaMemset(B.act_n, 0, sizeof(uint32_t)));
    CK(dalloc(&B.nact, 1));
    CK(dalloc(&B.frame, 1));
    CK(cudaMemset(B.nact, 0, sizeof(int32_t)));
    CK(cudaMemset(B.frame, 0, sizeof(int32_t)));
    c->stage_bytes = N * (sizeof(sphmp_display_pack) + sizeof(sphmp_calc_pack));
    if (c->stage_bytes < G * sizeof(int32_t)) c->stage_bytes = G * sizeof(int32_t);
    CK(cudaMalloc(&c->stage, c->stage_bytes));
    // zero everything the kernels may read before it is first written
    for (int f = 0; f < kNumFloat4Fields; f++)
        for (int b = 0; b < 2; b++) CK(cudaMemset(B.f4[f][b], 0, sizeof(float4) * N));
    CK(cudaMemset(B.densp, 0, sizeof(float2) * N));
    CK(cudaMemset(B.accel4, 0, sizeof(float4) * N));
    CK(cudaMemset(B.drift4, 0, sizeof(float4) * 3 * N));
    CK(cudaMemset(B.velxcor, 0, sizeof(float4) * N));
    CK(cudaMemset(B.pmod, 0, sizeof(float) * N));
    CK(cudaMemset(B.mgcell, 0xFF, sizeof(uint32_t) * N));
    CK(cudaMemset(B.opos, 0, sizeof(uint32_t) * N));
    CK(cudaMemset(B.oidx, 0, sizeof(uint32_t) * N));
    CK(cudaMemset(B.osrc, 0, sizeof(uint32_t) * N));
    CK(cudaMemset(B.midsort, 0, sizeof(uint32_t) * N));
    CK(cudaMemset(B.mgndx, 0xFF, sizeof(uint32_t) * N));
    CK(cudaMemset(B.mgridoff, 0, sizeof(int32_t) * G));
    CK(cudaMemset(B.mgridcnt, 0, sizeof(int32_t) * G));
    CK(cudaMemset(B.cstart, 0, sizeof(uint32_t) * (G + 2)));
    CK(cudaMemset(B.err, 0, sizeof(uint32_t)));
    CK(cudaMemset(B.color, 0, sizeof(float4) * N));
    CK(cudaMemset(B.bornid, 0, sizeof(int32_t) * N));
    CK(cudaMemset(B.mass_raw, 0, sizeof(float) * N));
    // cudaMemset runs on the legacy default stream, which the context's
    // non-blocking stream does not wait for: without this wait a first upload
    // or state copy could be overwritten by a zero fill that runs after it
    CK(cudaDeviceSynchronize());
    return SPHMP_OK;
}

// Read and clear the device error word; map the lowest set bit to a status.
sphmp_status take_device_errors(sphmp_ctx* c, uint32_t* bits_out) {
    uint32_t bits = 0;
    CK(cudaMemcpyAsync(&bits, c->B.err, sizeof(uint32_t), cudaMemcpyDeviceToHost, c->stream));
    CK(cudaMemsetAsync(c->B.err, 0, sizeof(uint32_t), c->stream));
    CK(cudaStreamSynchronize(c->stream));
    if (bits_out) *bits_out = bits;
    if (bits) {
        for (int s = 1; s < 32; s++)
            if (bits & (1u << s)) {
                const char* what = s == SPHMP_ERR_UNSUPPORTED_TYPE ? "particle type other than fluid (0) or boundary (1)"
                                   : s == SPHMP_ERR_NOT_FINITE     ? "non-finite particle position"
                                   : s == SPHMP_ERR_BAD_MASS       ? "fluid particle with mass <= 0 or not finite"
                                   : s == SPHMP_ERR_CELL_OVERFLOW  ? "a grid cell holds more than 8192 particles"
                                   : s == SPHMP_ERR_CAPACITY       ? "device-side emission reached the capacity"
                                   : s == SPHMP_ERR_TIMEOUT        ? "a tensor-core wait of the corrector ran out"
                                                                   : "device error";
                return fail((sphmp_status)s, "device reported: %s", what);
            }
    }
    return SPHMP_OK;
}

inline sphmp_status need_ctx(const sphmp_ctx* c) {
    if (!c) return fail(SPHMP_ERR_INVALID_ARG, "context is NULL");
    return SPHMP_OK;
}

inline sphmp_status need_grid(const sphmp_ctx* c) {
    if (!c->grid_valid) return fail(SPHMP_ERR_STATE, "no cell list for the current slot order (run the sort first)");
    return SPHMP_OK;
}

// The particle count after steps that may have emitted on the device.
sphmp_status refresh_n(sphmp_ctx* c) {
    if (!c->n_stale) return SPHMP_OK;
    int32_t n = 0;
    CK(cudaMemcpyAsync(&n, c->B.nact, sizeof(n), cudaMemcpyDeviceToHost, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    c->n = n;
    c->prm.num = n;
    c->n_stale = false;
    return SPHMP_OK;
}

inline void swap_all(sphmp_ctx* c) {
    for (int f = 0; f < kNumFloat4Fields; f++) c->cur[f] ^= 1;
}

// Density pass: the bucket kernel when the internal order of this sort is
// octant-grouped, otherwise the cell-search kernel; both write neighbour lists.
void run_density(sphmp_ctx* c, cudaStream_t s) {
    const DevParams P = dev_params(c);
    if (c->oct_valid) launch_density_oct(P, c->B, c->cur, s);
    else launch_density(P, c->B, c->cur, s);
    c->list_mode = 1;
    c->nbr_valid = true;
}

void run_force_drift(sphmp_ctx* c, bool force, bool drift, cudaStream_t s) {
    const DevParams P = dev_params(c);
    launch_force_drift(P, c->B, c->cur, force, drift, s);
}

// Optional event marks between the stages of a step (for sphmp_step_profile).
struct StageTimer {
    static constexpr int kMax = 24;
    cudaEvent_t ev[kMax + 1];
    const char* name[kMax];
    int n = 0;
    bool ok = true;
    StageTimer() {
        for (int i = 0; i <= kMax; i++)
            if (cudaEventCreate(&ev[i]) != cudaSuccess) ok = false;
    }
    ~StageTimer() {
        for (int i = 0; i <= kMax; i++) cudaEventDestroy(ev[i]);
    }
    void start(cudaStream_t s) { cudaEventRecord(ev[0], s); }
    void mark(cudaStream_t s, const char* nm) {
        if (n >= kMax) return;
        name[n] = nm;
        cudaEventRecord(ev[++n], s);
    }
};

// A corrected large step: the network and the step length it corrects.
struct LargeStep {
    sphmp_corrector* cor;
    float dt;
};

// Queue one full step on the context stream (no host synchronisation). With
// `L` (fused schedule only), the features are taken after the density pass and
// the network's correction is applied to the step's result.
sphmp_status enqueue_step(sphmp_ctx* c, int schedule, StageTimer* T = nullptr, const LargeStep* L = nullptr,
                          bool reuse_sorted = false) {
    const DevParams P = dev_params(c);
    const cudaStream_t s = c->stream;
    auto mark = [&](const char* nm) {
        if (T) T->mark(s, nm);
    };
    if (T) T->start(s);
    const bool reuse = reuse_sorted && c->sorted_dens_fresh && !c->emit_on;
    c->sorted_dens_fresh = false;
    if (!reuse) {
        if (c->emit_on) {
            launch_emit(P, c->B, c->cur, c->emitter, s);
            c->n_stale = true;
            mark("emit");
        }
        launch_hash(P, c->B, c->cur, s);
        mark("hash");
        c->hash_n = c->emit_on ? -1 : c->n;  // with an emitter the count is only known on the device
        launch_cell_starts(P, c->B, s);
        mark("cell_starts");
        launch_cell_order(P, c->B, c->cur, s);
        mark("cell_order");
        launch_rearrange(P, c->B, c->cur, false, s);
        mark("rearrange");
        swap_all(c);
        c->alpha_advanced = false;
        c->grid_valid = true;
        c->oct_valid = true;
        c->oct_built = false;
        c->nbr_valid = false;
        c->pos_sorted = true;
        run_density(c, s);
        mark("density");
    }
    const DevParams PL = dev_params(c);  // neighbour passes read the list
    if (schedule == SPHMP_SCHEDULE_FUSED) {
        if (L) {  // the force pass also fills the corrector's features
            const float* gv = c->prm.gravity;
            const float gabs = sqrtf(gv[0] * gv[0] + gv[1] * gv[1] + gv[2] * gv[2]);
            const float vs = sqrtf(fmaxf(gabs, 1e-3f) * c->prm.smoothradius);
            launch_force_drift_features(PL, c->B, c->cur, c->lfeat, c->lids, vs, L->dt, s);
            mark("force_drift_features");
        } else {
            run_force_drift(c, true, PL.multiphase != 0, s);
            mark("force_drift");
        }
        if (PL.st_on) {
            launch_surface_tension(PL, c->B, c->cur, s);
            mark("surface_tension");
        }
        launch_pass_c(PL, c->B, c->cur, s);
        mark(PL.multiphase ? "alpha_correct_advance" : "advance");
        swap_all(c);
        if (L) {
            CK(corrector_forward_on(L->cor, c->lfeat, PL.n, c->ly, c->B.err, s));
            launch_apply_correction(PL, c->B, c->cur, c->ly, corrector_out_scale(L->cor), c->lids, L->dt, c->lcorr, s);
            c->lrows = PL.n;
            mark("correction");
        }
        c->nbr_valid = false;  // positions moved
        c->oct_valid = false;
        c->pos_sorted = false;
    } else {
        if (PL.multiphase) {
            run_force_drift(c, false, true, s);
            mark("drift");
            launch_alpha_advance(PL, c->B, c->cur, s);
            mark("alpha_advance");
            c->cur[ALPHA] ^= 1;
            c->alpha_advanced = true;
            launch_correction(dev_params(c), c->B, c->cur, c->cur[ALPHA] ^ 1, s);
            mark("correction");
        }
        if (schedule == SPHMP_SCHEDULE_PROJECTU) {
            launch_force_projectu(PL, c->B, c->cur, c->cur[ALPHA] ^ 1, s);
            mark("force_projectu");
        } else {
            run_force_drift(c, true, false, s);
            mark("force");
        }
        if (PL.st_on) {
            launch_surface_tension(PL, c->B, c->cur, s);
            mark("surface_tension");
        }
        launch_advance(dev_params(c), c->B, c->cur, s);
        mark("advance");
        c->nbr_valid = false;
        c->oct_valid = false;
        c->pos_sorted = false;
    }
    CHECK_LAUNCH("step");
    return SPHMP_OK;
}

sphmp_status check_schedule(const sphmp_ctx* c, int schedule) {
    if (schedule != SPHMP_SCHEDULE_REFERENCE && schedule != SPHMP_SCHEDULE_FUSED &&
        schedule != SPHMP_SCHEDULE_PROJECTU)
        return fail(SPHMP_ERR_INVALID_ARG, "unknown schedule %d", schedule);
    if (schedule == SPHMP_SCHEDULE_PROJECTU && !c->prm.multiphase)
        return fail(SPHMP_ERR_INVALID_ARG, "the project-U schedule is the multiphase step (set multiphase = 1)");
    return SPHMP_OK;
}

int field_width(int field) {
    switch (field) {
        case SPHMP_F_POS: case SPHMP_F_VEL: case SPHMP_F_VELEVAL: case SPHMP_F_ACCEL:
        case SPHMP_F_ALPHA: case SPHMP_F_ALPHA_PRE: case SPHMP_F_APREV: case SPHMP_F_VELXCOR: return 3;
        case SPHMP_F_DRIFT: return 9;
        default: return 1;
    }
}

}  // namespace

sphmp_status sphmp::record_error(sphmp_status st, const char* msg) { return fail(st, "%s", msg); }

// ===========================================================================
// C ABI
// ===========================================================================

extern "C" {

const char* sphmp_last_error(void) { return g_err.c_str(); }

const char* sphmp_version(void) { return "sphmp 0.1 sm_103a"; }

// The cells in Z-order for the Morton cell order (uploaded once per grid shape).
sphmp_status ensure_cell_order(sphmp_ctx* c) {
    const sphmp_params& p = c->prm;
    if (p.cell_order != SPHMP_CELL_ORDER_MORTON) return SPHMP_OK;
    if (memcmp(c->corder_res, p.gridres, sizeof(c->corder_res)) == 0) return SPHMP_OK;
    const uint32_t rx = (uint32_t)p.gridres[0], ry = (uint32_t)p.gridres[1], rz = (uint32_t)p.gridres[2];
    std::vector<std::pair<uint64_t, uint32_t>> key((size_t)p.gridtotal);
    for (uint32_t y = 0; y < ry; y++)
        for (uint32_t z = 0; z < rz; z++)
            for (uint32_t x = 0; x < rx; x++) {
                const uint32_t cell = (y * rz + z) * rx + x;
                key[cell] = {morton_code(x, y, z), cell};
            }
    std::sort(key.begin(), key.end());
    std::vector<uint32_t> order(key.size());
    for (size_t i = 0; i < key.size(); i++) order[i] = key[i].second;
    CK(cudaMemcpyAsync(c->B.corder, order.data(), sizeof(uint32_t) * order.size(), cudaMemcpyHostToDevice, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    memcpy(c->corder_res, p.gridres, sizeof(c->corder_res));
    return SPHMP_OK;
}

sphmp_status sphmp_create(const sphmp_params* p, sphmp_ctx** out) {
    if (!out) return fail(SPHMP_ERR_INVALID_ARG, "out is NULL");
    *out = nullptr;
    sphmp_status st = validate_params(p);
    if (st) return st;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev <= 0) {
        cudaGetLastError();
        return fail(SPHMP_ERR_NO_DEVICE, "no CUDA device available");
    }
    sphmp_ctx* c = new sphmp_ctx();
    c->prm = *p;
    c->cap = p->maxNum;
    c->gcap = p->gridtotal;
    c->n = p->num;
    cudaGetDevice(&c->device);
    cudaError_t e = cudaStreamCreateWithFlags(&c->own_stream, cudaStreamNonBlocking);
    if (e != cudaSuccess) {
        delete c;
        return cuda_fail(e, "cudaStreamCreate");
    }
    c->stream = c->own_stream;
    st = alloc_buffers(c);
    if (st) {
        free_buffers(c);
        cudaStreamDestroy(c->own_stream);
        delete c;
        return st;
    }
    launch_set_count(c->B, c->n, c->stream);
    st = ensure_cell_order(c);
    if (st) {
        sphmp_destroy(c);
        return st;
    }
    *out = c;
    return SPHMP_OK;
}

sphmp_status sphmp_destroy(sphmp_ctx* c) {
    if (!c) return SPHMP_OK;
    cudaStreamSynchronize(c->stream);
    if (c->copy_stream) {
        cudaStreamSynchronize(c->copy_stream);
        cudaStreamDestroy(c->copy_stream);
    }
    for (int k = 0; k < 2; k++) {
        cudaFree(c->dl_stage[k]);
        if (c->dl_packed[k]) cudaEventDestroy(c->dl_packed[k]);
        if (c->dl_done[k]) cudaEventDestroy(c->dl_done[k]);
    }
    drop_graph(c);
    free_buffers(c);
    void* lbufs[] = {c->lfeat, c->lids, c->ly, c->lcorr, c->xstage, c->cmap, c->cred};
    for (void* q : lbufs) cudaFree(q);
    if (c->own_stream) cudaStreamDestroy(c->own_stream);
    delete c;
    return SPHMP_OK;
}

sphmp_status sphmp_set_params(sphmp_ctx* c, const sphmp_params* p) {
    if (sphmp_status st = need_ctx(c)) return st;
    if (sphmp_status st = validate_params(p)) return st;
    if (p->maxNum > c->cap) return fail(SPHMP_ERR_CAPACITY, "maxNum %d exceeds the allocated capacity %d", p->maxNum, c->cap);
    if (p->gridtotal > c->gcap) return fail(SPHMP_ERR_CAPACITY, "gridtotal %d exceeds the allocated %d cells", p->gridtotal, c->gcap);
    if (sphmp_status st = refresh_n(c)) return st;
    const bool grid_changed = memcmp(p->gridres, c->prm.gridres, sizeof(p->gridres)) != 0 ||
                              memcmp(p->gridmin, c->prm.gridmin, sizeof(p->gridmin)) != 0 ||
                              memcmp(p->gridIdfac, c->prm.gridIdfac, sizeof(p->gridIdfac)) != 0;
    // neighbour lists and the octant buckets hold for the radius they were built with
    const bool radius_changed = p->smoothradius != c->prm.smoothradius || p->simscale != c->prm.simscale;
    const bool order_changed = p->cell_order != c->prm.cell_order;
    c->prm = *p;
    c->prm.maxNum = c->cap;
    c->prm.num = c->n;
    if (sphmp_status st = ensure_cell_order(c)) return st;
    if (grid_changed || order_changed) c->grid_valid = false;
    if (grid_changed || radius_changed || order_changed) {
        c->nbr_valid = false;
        c->oct_valid = false;
    }
    drop_graph(c);
    return SPHMP_OK;
}

sphmp_status sphmp_get_params(const sphmp_ctx* c, sphmp_params* p) {
    if (sphmp_status st = need_ctx(c)) return st;
    if (!p) return fail(SPHMP_ERR_INVALID_ARG, "params is NULL");
    if (sphmp_status st = refresh_n(const_cast<sphmp_ctx*>(c))) return st;
    *p = c->prm;
    p->num = c->n;
    return SPHMP_OK;
}

sphmp_status sphmp_set_stream(sphmp_ctx* c, void* stream) {
    if (sphmp_status st = need_ctx(c)) return st;
    CK(cudaStreamSynchronize(c->stream));
    c->stream = stream ? (cudaStream_t)stream : c->own_stream;
    drop_graph(c);
    return SPHMP_OK;
}

sphmp_status sphmp_sync(sphmp_ctx* c) {
    if (sphmp_status st = need_ctx(c)) return st;
    CK(cudaStreamSynchronize(c->stream));
    if (sphmp_status st = refresh_n(c)) return st;
    if (c->copy_stream) CK(cudaStreamSynchronize(c->copy_stream));
    return take_device_errors(c, nullptr);
}

int32_t sphmp_num_particles(const sphmp_ctx* c) {
    if (!c) return 0;
    if (refresh_n(const_cast<sphmp_ctx*>(c))) return -1;
    return c->n;
}

sphmp_status sphmp_device_errors(sphmp_ctx* c, uint32_t* bits) {
    if (sphmp_status st = need_ctx(c)) return st;
    uint32_t b = 0;
    sphmp_status st = take_device_errors(c, &b);
    if (bits) *bits = b;
    return st == SPHMP_ERR_CUDA ? st : SPHMP_OK;
}

// ---- transfers ----

// Records [start, end) from the host, or (`staged`) already in the staging buffer.
static sphmp_status upload_records(sphmp_ctx* c, const sphmp_display_pack* disp, const sphmp_calc_pack* calc,
                                   int start, int end, bool staged = false) {
    if (!staged && (!disp || !calc)) return fail(SPHMP_ERR_INVALID_ARG, "record pointers are NULL");
    if (start < 0 || end < start) return fail(SPHMP_ERR_INVALID_ARG, "bad range [%d, %d)", start, end);
    if (end > c->cap) return fail(SPHMP_ERR_CAPACITY, "%d particles exceed the capacity %d", end, c->cap);
    const int m = end - start;
    auto* d_disp = reinterpret_cast<sphmp_display_pack*>(c->stage);
    auto* d_calc = reinterpret_cast<sphmp_calc_pack*>(reinterpret_cast<char*>(c->stage) +
                                                      sizeof(sphmp_display_pack) * (size_t)c->cap);
    if (take_device_errors(c, nullptr) == SPHMP_ERR_CUDA) return SPHMP_ERR_CUDA;  // clear stale bits
    if (m > 0 && !staged) {
        CK(cudaMemcpyAsync(d_disp, disp, sizeof(sphmp_display_pack) * (size_t)m, cudaMemcpyHostToDevice, c->stream));
        CK(cudaMemcpyAsync(d_calc, calc, sizeof(sphmp_calc_pack) * (size_t)m, cudaMemcpyHostToDevice, c->stream));
    }
    // a full upload rewrites every double-buffered field, so it can start from the
    // first buffer of each: the selectors are then those of a fresh context, and a
    // step captured after a fresh upload and the first sort serves again after this
    // upload and that sort (an append keeps the selectors of the particles before it)
    if (start == 0)
        for (int f = 0; f < kNumFloat4Fields; f++) c->cur[f] = 0;
    c->n = end;
    c->prm.num = end;
    c->n_stale = false;
    c->hash_n = -1;
    launch_set_count(c->B, end, c->stream);
    const DevParams P = dev_params(c);
    launch_unpack_aos(P, c->B, c->cur, d_disp, d_calc, start, end, c->stream);
    CHECK_LAUNCH("unpack records");
    c->alpha_advanced = false;
    c->grid_valid = false;
    c->nbr_valid = false;
    c->oct_valid = false;
    c->oct_built = false;
    c->pos_sorted = false;
    // a captured step serves any state of the same count and buffer selectors
    // (it starts with the sort and restores the selectors), so it survives an
    // upload of the same number of records; sphmp_step re-captures when the
    // count or a selector differs
    if (c->graph_n != (c->emit_on ? -2 : end)) drop_graph(c);
    CK(cudaStreamSynchronize(c->stream));
    return take_device_errors(c, nullptr);
}

sphmp_status sphmp_upload_aos(sphmp_ctx* c, const sphmp_display_pack* disp, const sphmp_calc_pack* calc, int32_t n) {
    if (sphmp_status st = need_ctx(c)) return st;
    if (n < 0) return fail(SPHMP_ERR_INVALID_ARG, "n < 0");
    return upload_records(c, disp, calc, 0, n);
}

sphmp_status sphmp_emit_aos(sphmp_ctx* c, const sphmp_display_pack* disp, const sphmp_calc_pack* calc,
                            int32_t start, int32_t end) {
    if (sphmp_status st = need_ctx(c)) return st;
    if (sphmp_status st = refresh_n(c)) return st;
    if (start != c->n) return fail(SPHMP_ERR_INVALID_ARG, "emission must append at slot %d (got start %d)", c->n, start);
    return upload_records(c, disp, calc, start, end);
}

sphmp_status sphmp_download_aos(sphmp_ctx* c, sphmp_display_pack* disp, sphmp_calc_pack* calc, int32_t n) {
    if (sphmp_status st = need_ctx(c)) return st;
    if (!disp) return fail(SPHMP_ERR_INVALID_ARG, "display pointer is NULL");
    if (sphmp_status st = refresh_n(c)) return st;
    if (n < 0 || n > c->n) return fail(SPHMP_ERR_CAPACITY, "n %d outside [0, %d]", n, c->n);
    auto* d_disp = reinterpret_cast<sphmp_display_pack*>(c->stage);
    auto* d_calc = calc ? reinterpret_cast<sphmp_calc_pack*>(reinterpret_cast<char*>(c->stage) +
                                                             sizeof(sphmp_display_pack) * (size_t)c->cap)
                        : nullptr;
    const DevParams P = dev_params(c);
    launch_pack_aos(P, c->B, c->cur, d_disp, d_calc, n, c->stream);
    CHECK_LAUNCH("pack records");
    if (n > 0) {
        CK(cudaMemcpyAsync(disp, d_disp, sizeof(sphmp_display_pack) * (size_t)n, cudaMemcpyDeviceToHost, c->stream));
        if (calc)
            CK(cudaMemcpyAsync(calc, d_calc, sizeof(sphmp_calc_pack) * (size_t)n, cudaMemcpyDeviceToHost, c->stream));
    }
    CK(cudaStreamSynchronize(c->stream));
    return SPHMP_OK;
}

sphmp_status sphmp_download_display_async(sphmp_ctx* c, sphmp_display_pack* disp, int32_t n) {
    if (sphmp_status st = need_ctx(c)) return st;
    if (!disp) return fail(SPHMP_ERR_INVALID_ARG, "display pointer is NULL");
    if (sphmp_status st = refresh_n(c)) return st;
    if (n < 0 || n > c->n) return fail(SPHMP_ERR_CAPACITY, "n %d outside [0, %d]", n, c->n);
    if (!c->copy_stream) {  // first use: the copy stream, two staging buffers and their events
        CK(cudaStreamCreateWithFlags(&c->copy_stream, cudaStreamNonBlocking));
        for (int k = 0; k < 2; k++) {
            CK(cudaMalloc(&c->dl_stage[k], sizeof(sphmp_display_pack) * (size_t)(c->cap > 0 ? c->cap : 1)));
            CK(cudaEventCreateWithFlags(&c->dl_packed[k], cudaEventDisableTiming));
            CK(cudaEventCreateWithFlags(&c->dl_done[k], cudaEventDisableTiming));
            CK(cudaEventRecord(c->dl_done[k], c->copy_stream));
        }
    }
    const int k = c->dl_next;
    c->dl_next ^= 1;
    // the staging buffer is free once the copy of two downloads ago has landed
    CK(cudaStreamWaitEvent(c->stream, c->dl_done[k], 0));
    launch_pack_aos(dev_params(c), c->B, c->cur, c->dl_stage[k], nullptr, n, c->stream);
    CHECK_LAUNCH("pack display records");
    CK(cudaEventRecord(c->dl_packed[k], c->stream));
    CK(cudaStreamWaitEvent(c->copy_stream, c->dl_packed[k], 0));
    if (n > 0)
        CK(cudaMemcpyAsync(disp, c->dl_stage[k], sizeof(sphmp_display_pack) * (size_t)n, cudaMemcpyDeviceToHost,
                           c->copy_stream));
    CK(cudaEventRecord(c->dl_done[k], c->copy_stream));
    return SPHMP_OK;
}

sphmp_status sphmp_download_wait(sphmp_ctx* c) {
    if (sphmp_status st = need_ctx(c)) return st;
    if (c->copy_stream) CK(cudaStreamSynchronize(c->copy_stream));
    return SPHMP_OK;
}

// Uploaded sort arrays are indexed with on the device: a cell id must be an
// interior cell (the neighbour loops visit its 3x3x3 block) or GRID_UNDEF, and
// the per-cell counts must be non-negative and add up to at most n.
static sphmp_status check_sort_upload(const sphmp_ctx* c, int field, const void* host, int32_t n) {
    const sphmp_params& p = c->prm;
    if (field == SPHMP_F_MGCELL) {
        const uint32_t* v = static_cast<const uint32_t*>(host);
        for (int32_t i = 0; i < n; i++) {
            if (v[i] == SPHMP_GRID_UNDEF) continue;
            const uint32_t x = v[i] % (uint32_t)p.gridres[0], yz = v[i] / (uint32_t)p.gridres[0];
            const uint32_t z = yz % (uint32_t)p.gridres[2], y = yz / (uint32_t)p.gridres[2];
            if (v[i] >= (uint32_t)p.gridtotal || x < 1 || x + 2 > (uint32_t)p.gridres[0] || z < 1 ||
                z + 2 > (uint32_t)p.gridres[2] || y < 1 || y + 2 > (uint32_t)p.gridres[1])
                return fail(SPHMP_ERR_INVALID_ARG, "mgcell[%d] = %u is not an interior cell of the grid", i, v[i]);
        }
    } else if (field == SPHMP_F_MGRIDCNT) {
        const int32_t* v = static_cast<const int32_t*>(host);
        int64_t sum = 0;
        for (int32_t i = 0; i < n; i++) {
            if (v[i] < 0) return fail(SPHMP_ERR_INVALID_ARG, "mgridcnt[%d] = %d < 0", i, v[i]);
            sum += v[i];
        }
        if (sum > c->n) return fail(SPHMP_ERR_INVALID_ARG, "mgridcnt adds up to %lld > %d particles", (long long)sum, c->n);
    }
    return SPHMP_OK;
}

static void* sort_array(sphmp_ctx* c, int field, size_t* count) {
    switch (field) {
        case SPHMP_F_MGCELL: *count = c->n; return c->B.mgcell;
        case SPHMP_F_MIDSORT: *count = c->n; return c->B.midsort;
        case SPHMP_F_MGNDX: *count = c->n; return c->B.mgndx;
        case SPHMP_F_MGRIDOFF: *count = c->prm.gridtotal; return c->B.mgridoff;
        case SPHMP_F_MGRIDCNT: *count = c->prm.gridtotal; return c->B.mgridcnt;
        default: return nullptr;
    }
}

sphmp_status sphmp_download_field(sphmp_ctx* c, int32_t field, void* host, int32_t n) {
    if (sphmp_status st = need_ctx(c)) return st;
    if (!host) return fail(SPHMP_ERR_INVALID_ARG, "host pointer is NULL");
    if (field < 0 || field >= SPHMP_F_COUNT) return fail(SPHMP_ERR_INVALID_ARG, "unknown field %d", field);
    if (sphmp_status st = refresh_n(c)) return st;
    size_t count = 0;
    if (void* arr = sort_array(c, field, &count)) {
        if (n < 0 || (size_t)n > count) return fail(SPHMP_ERR_CAPACITY, "n %d exceeds %zu entries", n, count);
        CK(cudaMemcpyAsync(host, arr, sizeof(uint32_t) * (size_t)n, cudaMemcpyDeviceToHost, c->stream));
        CK(cudaStreamSynchronize(c->stream));
        return SPHMP_OK;
    }
    if (n < 0 || n > c->n) return fail(SPHMP_ERR_CAPACITY, "n %d outside [0, %d]", n, c->n);
    const int a_cur = c->cur[ALPHA];
    const int a_pre = c->alpha_advanced ? a_cur ^ 1 : a_cur;
    const DevParams P = dev_params(c);
    launch_pack_field(P, c->B, c->cur, field, a_cur, a_pre, c->stage, n, c->stream);
    CHECK_LAUNCH("pack field");
    CK(cudaMemcpyAsync(host, c->stage, sizeof(float) * (size_t)field_width(field) * n, cudaMemcpyDeviceToHost, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    return SPHMP_OK;
}

// A per-particle field (slot order, n entries) from device memory `dev` into the state.
static sphmp_status unpack_field_staged(sphmp_ctx* c, int field, const void* dev, int n) {
    if (field == SPHMP_F_ALPHA && !c->alpha_advanced) {
        // keep the start-of-step fractions in the other buffer, then overwrite the current ones
        CK(cudaMemcpyAsync(c->B.f4[ALPHA][c->cur[ALPHA] ^ 1], c->B.f4[ALPHA][c->cur[ALPHA]],
                           sizeof(float4) * (size_t)c->cap, cudaMemcpyDeviceToDevice, c->stream));
        c->cur[ALPHA] ^= 1;
        CK(cudaMemcpyAsync(c->B.f4[ALPHA][c->cur[ALPHA]], c->B.f4[ALPHA][c->cur[ALPHA] ^ 1],
                           sizeof(float4) * (size_t)c->cap, cudaMemcpyDeviceToDevice, c->stream));
        c->alpha_advanced = true;
    }
    const int a_cur = c->cur[ALPHA];
    const int a_pre = c->alpha_advanced ? a_cur ^ 1 : a_cur;
    const DevParams P = dev_params(c);
    launch_unpack_field(P, c->B, c->cur, field, a_cur, a_pre, dev, n, c->stream);
    CHECK_LAUNCH("unpack field");
    if (field == SPHMP_F_POS) {
        c->nbr_valid = false;
        c->oct_valid = false;
        c->oct_built = false;
        c->pos_sorted = false;
    }
    drop_graph(c);
    CK(cudaStreamSynchronize(c->stream));
    return SPHMP_OK;
}

sphmp_status sphmp_upload_field(sphmp_ctx* c, int32_t field, const void* host, int32_t n) {
    if (sphmp_status st = need_ctx(c)) return st;
    if (!host) return fail(SPHMP_ERR_INVALID_ARG, "host pointer is NULL");
    if (field < 0 || field >= SPHMP_F_COUNT) return fail(SPHMP_ERR_INVALID_ARG, "unknown field %d", field);
    if (sphmp_status st = refresh_n(c)) return st;
    if (field == SPHMP_F_DENS || field == SPHMP_F_TYPE || field == SPHMP_F_MASS || field == SPHMP_F_BORNID ||
        field == SPHMP_F_VELXCOR)
        return fail(SPHMP_ERR_INVALID_ARG, "field %d is download-only (upload it with sphmp_upload_aos)", field);
    size_t count = 0;
    if (void* arr = sort_array(c, field, &count)) {
        if (c->prm.cell_order != SPHMP_CELL_ORDER_LINEAR)
            return fail(SPHMP_ERR_STATE, "sort arrays can be uploaded only in the linear cell order");
        if (n < 0 || (size_t)n > count) return fail(SPHMP_ERR_CAPACITY, "n %d exceeds %zu entries", n, count);
        if (sphmp_status st = check_sort_upload(c, field, host, n)) return st;
        CK(cudaMemcpyAsync(arr, host, sizeof(uint32_t) * (size_t)n, cudaMemcpyHostToDevice, c->stream));
        c->nbr_valid = false;
        c->oct_valid = false;
        c->oct_built = false;
        c->pos_sorted = false;
        if (field == SPHMP_F_MGRIDCNT) {
            // rebuild the cell starts (and mgridoff) from the uploaded counts
            CK(cudaMemcpyAsync(c->B.ccount, c->B.mgridcnt, sizeof(uint32_t) * (size_t)c->prm.gridtotal,
                               cudaMemcpyDeviceToDevice, c->stream));
            DevParams P = dev_params(c);
            const int saved = P.n;
            P.n = 0;  // scan only: no scatter / cell sort
            launch_grid_list(P, c->B, c->cur, c->stream);
            P.n = saved;
            // cstart[G+1] must still be n
            const uint32_t nn = (uint32_t)c->n;
            CK(cudaMemcpyAsync(c->B.cstart + c->prm.gridtotal + 1, &nn, sizeof(uint32_t), cudaMemcpyHostToDevice, c->stream));
            CHECK_LAUNCH("rebuild cell starts");
            c->grid_valid = true;
        }
        drop_graph(c);
        CK(cudaStreamSynchronize(c->stream));
        return SPHMP_OK;
    }
    if (n < 0 || n > c->n) return fail(SPHMP_ERR_CAPACITY, "n %d outside [0, %d]", n, c->n);
    CK(cudaMemcpyAsync(c->stage, host, sizeof(float) * (size_t)field_width(field) * n, cudaMemcpyHostToDevice, c->stream));
    return unpack_field_staged(c, field, c->stage, n);
}

// ---- per-pass entry points ----

sphmp_status sphmp_get_particle_index(sphmp_ctx* c) {
    if (sphmp_status st = need_ctx(c)) return st;
    if (sphmp_status st = refresh_n(c)) return st;
    launch_hash(dev_params(c), c->B, c->cur, c->stream);
    CHECK_LAUNCH("GetParticleIndex");
    c->hash_n = c->n;
    c->grid_valid = false;
    c->nbr_valid = false;
    c->oct_valid = false;
    c->oct_built = false;
    return SPHMP_OK;
}

sphmp_status sphmp_get_grid_list(sphmp_ctx* c) {
    if (sphmp_status st = need_ctx(c)) return st;
    if (sphmp_status st = refresh_n(c)) return st;
    // the scatter places every slot by its cell key and rank: both must exist for the current count
    if (c->hash_n != c->n)
        return fail(SPHMP_ERR_STATE, "no cell keys for the current %d particles (run GetParticleIndex first)", c->n);
    launch_grid_list(dev_params(c), c->B, c->cur, c->stream);
    CHECK_LAUNCH("GetGridList");
    c->oct_built = true;
    return SPHMP_OK;
}

sphmp_status sphmp_rearrange_data(sphmp_ctx* c) {
    if (sphmp_status st = need_ctx(c)) return st;
    // without this library's grid list (sort arrays uploaded by the caller) the
    // new internal order is the plain sorted slot order
    launch_rearrange(dev_params(c), c->B, c->cur, !c->oct_built, c->stream);
    CHECK_LAUNCH("RearrageData");
    swap_all(c);
    c->alpha_advanced = false;
    c->grid_valid = true;
    c->nbr_valid = false;
    c->oct_valid = c->oct_built;
    c->oct_built = false;
    c->pos_sorted = true;
    return SPHMP_OK;
}

sphmp_status sphmp_compute_boundary_density(sphmp_ctx* c) {
    if (sphmp_status st = need_ctx(c)) return st;
    if (sphmp_status st = need_grid(c)) return st;
    launch_boundary_volume(dev_params(c), c->B, c->cur, c->stream);
    CHECK_LAUNCH("ComputeBoundaryDensity");
    c->nbr_valid = false;
    return SPHMP_OK;
}

sphmp_status sphmp_compute_pressure(sphmp_ctx* c) {
    if (sphmp_status st = need_ctx(c)) return st;
    if (sphmp_status st = need_grid(c)) return st;
    run_density(c, c->stream);
    CHECK_LAUNCH("MfComputePressure");
    return SPHMP_OK;
}

sphmp_status sphmp_compute_drift_vel(sphmp_ctx* c) {
    if (sphmp_status st = need_ctx(c)) return st;
    if (sphmp_status st = need_grid(c)) return st;
    run_force_drift(c, false, true, c->stream);
    CHECK_LAUNCH("MfComputeDriftVel");
    return SPHMP_OK;
}

sphmp_status sphmp_compute_alpha_advance(sphmp_ctx* c) {
    if (sphmp_status st = need_ctx(c)) return st;
    if (sphmp_status st = need_grid(c)) return st;
    if (c->alpha_advanced)
        return fail(SPHMP_ERR_STATE, "volume fractions already advanced in this step (re-sort first)");
    launch_alpha_advance(dev_params(c), c->B, c->cur, c->stream);
    CHECK_LAUNCH("MfComputeAlphaAdvance");
    c->cur[ALPHA] ^= 1;
    c->alpha_advanced = true;
    return SPHMP_OK;
}

sphmp_status sphmp_compute_correction(sphmp_ctx* c) {
    if (sphmp_status st = need_ctx(c)) return st;
    const int pre = c->alpha_advanced ? c->cur[ALPHA] ^ 1 : c->cur[ALPHA];
    launch_correction(dev_params(c), c->B, c->cur, pre, c->stream);
    CHECK_LAUNCH("MfComputeCorrection");
    return SPHMP_OK;
}

sphmp_status sphmp_compute_force(sphmp_ctx* c) {
    if (sphmp_status st = need_ctx(c)) return st;
    if (sphmp_status st = need_grid(c)) return st;
    const DevParams P = dev_params(c);
    run_force_drift(c, true, false, c->stream);
    if (P.st_on) launch_surface_tension(P, c->B, c->cur, c->stream);
    CHECK_LAUNCH("MfComputeForce");
    return SPHMP_OK;
}

sphmp_status sphmp_compute_force_projectu(sphmp_ctx* c) {
    if (sphmp_status st = need_ctx(c)) return st;
    if (sphmp_status st = need_grid(c)) return st;
    const DevParams P = dev_params(c);
    const int pre = c->alpha_advanced ? c->cur[ALPHA] ^ 1 : c->cur[ALPHA];
    launch_force_projectu(P, c->B, c->cur, pre, c->stream);
    if (P.st_on) launch_surface_tension(P, c->B, c->cur, c->stream);
    CHECK_LAUNCH("ComputeForce_projectu");
    return SPHMP_OK;
}

sphmp_status sphmp_set_device_emitter(sphmp_ctx* c, const sphmp_emitter* e, int32_t layers, int32_t phase,
                                      int32_t interval, float jitter, uint64_t seed) {
    if (sphmp_status st = need_ctx(c)) return st;
    if (sphmp_status st = refresh_n(c)) return st;
    if (!e || interval <= 0) {
        c->emit_on = false;
        drop_graph(c);
        return SPHMP_OK;
    }
    if (!(e->spacing > 0.0f) || !(e->radius >= 0.0f) || layers < 0 || phase < 0 || phase >= SPHMP_MAX_PHASES)
        return fail(SPHMP_ERR_INVALID_ARG, "emitter needs spacing > 0, radius >= 0, layers >= 0, phase in [0, 3)");
    const double side = 2.0 * (double)(int)(e->radius / e->spacing) + 1.0;
    if (side * side * (double)layers > 1.0e9)
        return fail(SPHMP_ERR_INVALID_ARG, "emitter has %.3g lattice sites per emission (at most 1e9)",
                    side * side * (double)layers);
    const sphmp_params& p = c->prm;
    if (!(p.massArr[phase] > 0.0f) || !isfinite(p.massArr[phase]))
        return fail(SPHMP_ERR_BAD_MASS, "phase %d has mass %g (massArr)", phase, (double)p.massArr[phase]);
    DevEmitter E{};
    emit_rotation(e->dir, E.rot);
    for (int a = 0; a < 3; a++) {
        E.pos[a] = e->position[a];
        E.dir[a] = e->dir[a];
    }
    E.vel = e->vel;
    E.radius = e->radius;
    E.spacing = e->spacing;
    E.jitter = jitter;
    E.mass = p.massArr[phase];
    E.restdens = p.densArr[phase];
    E.visc = p.viscArr[phase];
    E.seed = seed;
    E.res = (int)(e->radius / e->spacing);
    E.layers = layers;
    E.interval = interval;
    E.onehot = 0;  // sphmp_upload_aos's rule: the first phase with this rest density
    for (int k = 0; k < p.nphase; k++)
        if (p.densArr[k] == E.restdens) {
            E.onehot = k;
            break;
        }
    c->emitter = E;
    c->emit_on = true;
    drop_graph(c);
    CK(cudaMemsetAsync(c->B.frame, 0, sizeof(int32_t), c->stream));
    return SPHMP_OK;
}

sphmp_status sphmp_advance(sphmp_ctx* c) {
    if (sphmp_status st = need_ctx(c)) return st;
    launch_advance(dev_params(c), c->B, c->cur, c->stream);
    CHECK_LAUNCH("MfAdvance");
    c->nbr_valid = false;
    c->oct_valid = false;
    c->pos_sorted = false;
    return SPHMP_OK;
}

// ---- launch-shape autotuner ----

static sphmp_status clone_state(sphmp_ctx* dst, sphmp_ctx* src);

sphmp_status sphmp_autotune(sphmp_ctx* c, int32_t trial_steps, int32_t allow_reorder, sphmp_tuning* out) {
    if (sphmp_status st = need_ctx(c)) return st;
    if (!out || trial_steps < 1) return fail(SPHMP_ERR_INVALID_ARG, "need an output and trial_steps >= 1");
    if (c->emit_on) return fail(SPHMP_ERR_STATE, "autotune a context without a device emitter");
    if (sphmp_status st = refresh_n(c)) return st;
    CK(cudaStreamSynchronize(c->stream));
    sphmp_params base = c->prm;
    base.num = c->n;
    base.maxNum = c->cap;
    base.gridtotal = c->prm.gridtotal;
    sphmp_ctx* t = nullptr;
    if (sphmp_status st = sphmp_create(&base, &t)) return st;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    sphmp_status st = SPHMP_OK;
    if (cudaEventCreate(&e0) != cudaSuccess || cudaEventCreate(&e1) != cudaSuccess)
        st = fail(SPHMP_ERR_CUDA, "cudaEventCreate failed");
    struct Cand {
        int order, window, heavy;
    };
    std::vector<Cand> cands;
    const int orders[2] = {SPHMP_CELL_ORDER_LINEAR, SPHMP_CELL_ORDER_MORTON};
    for (int o = 0; o < (allow_reorder ? 2 : 1); o++)
        for (int w : {16, 32})
            for (int h : {64, 128, 256}) cands.push_back({orders[o], w, h});
    // the context's own configuration first: its time is ms_before
    const Cand cur = {c->prm.cell_order, c->prm.bucket_window ? c->prm.bucket_window : (int)kBucketWindow,
                      c->prm.heavy_list ? c->prm.heavy_list : (int)kHeavyList};
    cands.insert(cands.begin(), cur);
    float best = 0.f;
    Cand pick = cur;
    int trials = 0;
    for (size_t k = 0; k < cands.size() && st == SPHMP_OK; k++) {
        sphmp_params q = base;
        q.cell_order = cands[k].order;
        q.bucket_window = cands[k].window;
        q.heavy_list = cands[k].heavy;
        if ((st = sphmp_set_params(t, &q))) break;
        if ((st = clone_state(t, c))) break;
        if ((st = sphmp_step(t, 1, SPHMP_SCHEDULE_FUSED, 1))) break;  // captures the graph
        if ((st = clone_state(t, c))) break;
        if ((st = sphmp_step(t, 1, SPHMP_SCHEDULE_FUSED, 1))) break;  // a warm replay from the same state
        if ((st = clone_state(t, c))) break;
        cudaEventRecord(e0, t->stream);
        if ((st = sphmp_step(t, trial_steps, SPHMP_SCHEDULE_FUSED, 1))) break;
        cudaEventRecord(e1, t->stream);
        if (cudaEventSynchronize(e1) != cudaSuccess) {
            st = fail(SPHMP_ERR_CUDA, "autotune timing failed");
            break;
        }
        float ms = 0.f;
        cudaEventElapsedTime(&ms, e0, e1);
        ms /= (float)trial_steps;
        trials++;
        if (k == 0) out->ms_before = ms;
        if (k == 0 || ms < best) {
            best = ms;
            pick = cands[k];
        }
    }
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    sphmp_destroy(t);
    if (st) return st;
    sphmp_params chosen = c->prm;
    chosen.cell_order = pick.order;
    chosen.bucket_window = pick.window;
    chosen.heavy_list = pick.heavy;
    if (sphmp_status s2 = sphmp_set_params(c, &chosen)) return s2;
    out->cell_order = pick.order;
    out->bucket_window = pick.window;
    out->heavy_list = pick.heavy;
    out->trials = trials;
    out->ms_per_step = best;
    return SPHMP_OK;
}

// ---- IISPH (fluid_system_host.cu:504-557, kernels in sphmp_iisph.cu) ----

sphmp_status sphmp_iisph_density(sphmp_ctx* c) {
    if (sphmp_status st = need_ctx(c)) return st;
    if (sphmp_status st = need_grid(c)) return st;
    launch_iisph_density(dev_params(c), c->B, c->cur, c->stream);
    CHECK_LAUNCH("ComputeDensityIISPH");
    return SPHMP_OK;
}

sphmp_status sphmp_iisph_predict_advection(sphmp_ctx* c) {
    if (sphmp_status st = need_ctx(c)) return st;
    if (sphmp_status st = need_grid(c)) return st;
    launch_iisph_predict(dev_params(c), c->B, c->cur, c->stream);
    CHECK_LAUNCH("PredictAdvection");
    return SPHMP_OK;
}

sphmp_status sphmp_iisph_pressure_iteration(sphmp_ctx* c, double* residue) {
    if (sphmp_status st = need_ctx(c)) return st;
    if (sphmp_status st = need_grid(c)) return st;
    if (sphmp_status st = refresh_n(c)) return st;
    launch_iisph_iteration(dev_params(c), c->B, c->cur, c->stream);
    CHECK_LAUNCH("Pressure_DP / Pressure_Iter");
    double red[3];
    CK(cudaMemcpyAsync(red, c->B.red + 8, sizeof(red), cudaMemcpyDeviceToHost, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    if (residue) {
        residue[0] = c->n > 0 ? red[0] / c->n : 0.0;      // the reference's quantity: sum / pnum
        residue[1] = red[2] > 0 ? red[1] / red[2] : 0.0;  // mean |residue| over in-grid fluid particles
    }
    return SPHMP_OK;
}

sphmp_status sphmp_iisph_pressure_solve(sphmp_ctx* c, float tol, int32_t min_iter, int32_t max_iter,
                                        int32_t* iters, double* residue) {
    if (sphmp_status st = need_ctx(c)) return st;
    if (!(tol >= 0.f) || min_iter < 0 || max_iter < 1 || min_iter > max_iter)
        return fail(SPHMP_ERR_INVALID_ARG, "need tol >= 0 and 0 <= min_iter <= max_iter, max_iter >= 1");
    double r[2] = {0.0, 0.0};
    int it = 0;
    while (it < max_iter) {
        if (sphmp_status st = sphmp_iisph_pressure_iteration(c, r)) return st;
        it++;
        if (it >= min_iter && r[1] <= (double)tol) break;
    }
    if (iters) *iters = it;
    if (residue) {
        residue[0] = r[0];
        residue[1] = r[1];
    }
    return SPHMP_OK;
}

sphmp_status sphmp_iisph_integrate(sphmp_ctx* c) {
    if (sphmp_status st = need_ctx(c)) return st;
    if (sphmp_status st = need_grid(c)) return st;
    launch_iisph_integrate(dev_params(c), c->B, c->cur, c->stream);
    CHECK_LAUNCH("IntegrateIISPH");
    c->nbr_valid = false;
    c->oct_valid = false;
    c->pos_sorted = false;
    return SPHMP_OK;
}

sphmp_status sphmp_step_iisph(sphmp_ctx* c, int32_t nsteps, float tol, int32_t max_iter, int32_t* iters,
                              double* residue) {
    if (sphmp_status st = need_ctx(c)) return st;
    if (nsteps < 0) return fail(SPHMP_ERR_INVALID_ARG, "nsteps < 0");
    for (int k = 0; k < nsteps; k++) {
        // RunIISPH (fluid_system.cpp:567-588) with its Integration call, which the reference comments out
        if (sphmp_status st = sphmp_get_particle_index(c)) return st;
        if (sphmp_status st = sphmp_get_grid_list(c)) return st;
        if (sphmp_status st = sphmp_rearrange_data(c)) return st;
        if (sphmp_status st = sphmp_iisph_density(c)) return st;
        if (sphmp_status st = sphmp_iisph_predict_advection(c)) return st;
        int32_t it = 0;
        if (sphmp_status st = sphmp_iisph_pressure_solve(c, tol, 2, max_iter, &it, residue)) return st;
        if (iters) iters[k] = it;
        if (sphmp_status st = sphmp_iisph_integrate(c)) return st;
    }
    CK(cudaStreamSynchronize(c->stream));
    return SPHMP_OK;
}

sphmp_status sphmp_step(sphmp_ctx* c, int32_t nsteps, int32_t schedule, int32_t use_graph) {
    if (sphmp_status st = need_ctx(c)) return st;
    if (nsteps < 0) return fail(SPHMP_ERR_INVALID_ARG, "nsteps < 0");
    if (sphmp_status st = check_schedule(c, schedule)) return st;
    if (nsteps == 0) return SPHMP_OK;
    // A fused step leaves every double buffer where it found it, so one captured
    // step replays for all later steps. The reference and project-U schedules flip
    // every buffer an odd number of times per step, so their graph holds two
    // steps; an odd remainder runs eagerly.
    const int per = schedule == SPHMP_SCHEDULE_FUSED ? 1 : 2;
    if (use_graph && nsteps >= per) {
        // with a device emitter the graph runs over the capacity and serves any count
        const int key = c->emit_on ? -2 : c->n;
        // the graph reads and writes the buffers selected at capture: any host call
        // that flipped a selector an odd number of times since (an eager step of
        // the reference order, a per-pass call, the sort before the first step)
        // needs a new capture
        if (!c->graph || c->graph_n != key || c->graph_schedule != schedule ||
            memcmp(c->graph_cur, c->cur, sizeof(c->graph_cur)) != 0) {
            drop_graph(c);
            cudaStream_t cap = c->stream;
            CK(cudaStreamBeginCapture(cap, cudaStreamCaptureModeThreadLocal));
            int saved[kNumFloat4Fields];
            memcpy(saved, c->cur, sizeof(saved));
            sphmp_status st = SPHMP_OK;
            for (int k = 0; k < per && !st; k++) st = enqueue_step(c, schedule);
            cudaGraph_t g = nullptr;
            cudaError_t e = cudaStreamEndCapture(cap, &g);
            if (st) {
                if (g) cudaGraphDestroy(g);
                return st;
            }
            if (e != cudaSuccess) return cuda_fail(e, "cudaStreamEndCapture");
            if (memcmp(saved, c->cur, sizeof(saved)) != 0) {
                cudaGraphDestroy(g);
                return fail(SPHMP_ERR_STATE, "internal: captured steps did not restore buffer selectors");
            }
            e = cudaGraphInstantiate(&c->graph, g, 0);
            cudaGraphDestroy(g);
            if (e != cudaSuccess) {
                c->graph = nullptr;
                return cuda_fail(e, "cudaGraphInstantiate");
            }
            c->graph_n = key;
            c->graph_schedule = schedule;
            memcpy(c->graph_cur, c->cur, sizeof(c->graph_cur));
        }
        for (int t = 0; t + per <= nsteps; t += per) CK(cudaGraphLaunch(c->graph, c->stream));
        if (c->emit_on) c->n_stale = true;
        // the state a step leaves behind (as enqueue_step sets it)
        c->alpha_advanced = schedule != SPHMP_SCHEDULE_FUSED && c->prm.multiphase;
        c->grid_valid = true;
        c->nbr_valid = false;
        c->oct_valid = false;
        c->oct_built = false;
        c->pos_sorted = false;
        c->list_mode = 1;
        c->hash_n = c->emit_on ? -1 : c->n;
        for (int t = 0; t < nsteps % per; t++)
            if (sphmp_status st = enqueue_step(c, schedule)) return st;
        return SPHMP_OK;
    }
    for (int t = 0; t < nsteps; t++)
        if (sphmp_status st = enqueue_step(c, schedule)) return st;
    return SPHMP_OK;
}

int32_t sphmp_step_profile(sphmp_ctx* c, int32_t schedule, float* ms, char* names, int32_t nmax) {
    if (need_ctx(c) != SPHMP_OK) return -SPHMP_ERR_INVALID_ARG;
    if (!ms || nmax <= 0) {
        fail(SPHMP_ERR_INVALID_ARG, "need an output array");
        return -SPHMP_ERR_INVALID_ARG;
    }
    if (sphmp_status st = check_schedule(c, schedule)) return -st;
    StageTimer T;
    if (!T.ok) {
        fail(SPHMP_ERR_CUDA, "cudaEventCreate failed");
        return -SPHMP_ERR_CUDA;
    }
    sphmp_status st = enqueue_step(c, schedule, &T);
    if (st) return -st;
    cudaError_t e = cudaStreamSynchronize(c->stream);
    if (e != cudaSuccess) return -cuda_fail(e, "cudaStreamSynchronize");
    const int n = T.n < nmax ? T.n : nmax;
    for (int i = 0; i < n; i++) {
        float t = 0.f;
        cudaEventElapsedTime(&t, T.ev[i], T.ev[i + 1]);
        ms[i] = t;
        if (names) {
            strncpy(names + 32 * i, T.name[i], 31);
            names[32 * i + 31] = 0;
        }
    }
    return n;
}

sphmp_status sphmp_step_large(sphmp_ctx* c, sphmp_corrector* cor, int32_t factor, int32_t nsteps) {
    if (sphmp_status st = need_ctx(c)) return st;
    if (factor < 1 || nsteps < 0) return fail(SPHMP_ERR_INVALID_ARG, "factor must be >= 1 and nsteps >= 0");
    if (cor && corrector_device(cor) != c->device)
        return fail(SPHMP_ERR_INVALID_ARG, "the corrector lives on another device");
    if (nsteps == 0) return SPHMP_OK;
    if (cor && !c->lfeat) {
        const size_t N = (size_t)c->cap;
        CK(cudaMalloc(&c->lfeat, sizeof(float) * SPHMP_LC_FEATURES * N));
        CK(cudaMalloc(&c->lids, sizeof(int32_t) * N));
        CK(cudaMalloc(&c->ly, sizeof(float) * 4 * N));
        CK(cudaMalloc(&c->lcorr, sizeof(float) * 4 * N));
    }
    const float dt0 = c->prm.dt;
    c->prm.dt = dt0 * (float)factor;
    const LargeStep L{cor, c->prm.dt};
    sphmp_status st = SPHMP_OK;
    for (int t = 0; t < nsteps && !st; t++)
        st = enqueue_step(c, SPHMP_SCHEDULE_FUSED, nullptr, cor ? &L : nullptr, t == 0);
    c->prm.dt = dt0;
    return st;
}

sphmp_status sphmp_learned_features(sphmp_ctx* c, float* feat, int32_t* ids, float* corr, int32_t* count) {
    if (sphmp_status st = need_ctx(c)) return st;
    if (!c->lfeat || c->lrows <= 0) return fail(SPHMP_ERR_STATE, "no corrected large step has run");
    const size_t n = (size_t)c->lrows;
    if (feat) CK(cudaMemcpyAsync(feat, c->lfeat, sizeof(float) * SPHMP_LC_FEATURES * n, cudaMemcpyDeviceToDevice, c->stream));
    if (ids) CK(cudaMemcpyAsync(ids, c->lids, sizeof(int32_t) * n, cudaMemcpyDeviceToDevice, c->stream));
    if (corr) CK(cudaMemcpyAsync(corr, c->lcorr, sizeof(float) * 4 * n, cudaMemcpyDeviceToDevice, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    if (count) *count = c->lrows;
    return take_device_errors(c, nullptr);
}

sphmp_status sphmp_copy_state(sphmp_ctx* dst, sphmp_ctx* src) {
    if (!dst || !src) return fail(SPHMP_ERR_INVALID_ARG, "context is NULL");
    if (dst == src) return fail(SPHMP_ERR_INVALID_ARG, "source and destination are the same context");
    if (dst->device != src->device) return fail(SPHMP_ERR_INVALID_ARG, "contexts on different devices");
    if (dst->prm.nphase != src->prm.nphase) return fail(SPHMP_ERR_INVALID_ARG, "phase counts differ");
    if (sphmp_status st = refresh_n(src)) return st;
    const int n = src->n;
    if (n > dst->cap) return fail(SPHMP_ERR_CAPACITY, "%d particles exceed the destination's capacity %d", n, dst->cap);
    if (!dst->xstage) CK(cudaMalloc(&dst->xstage, sizeof(float) * 6 * (size_t)(dst->cap > 0 ? dst->cap : 1)));
    CK(cudaStreamSynchronize(dst->stream));  // the destination's staging buffers are idle
    auto* d_disp = reinterpret_cast<sphmp_display_pack*>(dst->stage);
    auto* d_calc = reinterpret_cast<sphmp_calc_pack*>(reinterpret_cast<char*>(dst->stage) +
                                                      sizeof(sphmp_display_pack) * (size_t)dst->cap);
    float* xa = static_cast<float*>(dst->xstage);
    float* xg = xa + 3 * (size_t)dst->cap;
    // what sphmp_save_state writes: the records in slot order, the fractions, g - a
    const DevParams PS = dev_params(src);
    const int a_cur = src->cur[ALPHA];
    const int a_pre = src->alpha_advanced ? a_cur ^ 1 : a_cur;
    launch_pack_aos(PS, src->B, src->cur, d_disp, d_calc, n, src->stream);
    launch_pack_field(PS, src->B, src->cur, SPHMP_F_ALPHA, a_cur, a_pre, xa, n, src->stream);
    launch_pack_field(PS, src->B, src->cur, SPHMP_F_APREV, a_cur, a_pre, xg, n, src->stream);
    CHECK_LAUNCH("pack state");
    CK(cudaStreamSynchronize(src->stream));
    // what sphmp_load_state does with them
    if (sphmp_status st = upload_records(dst, nullptr, nullptr, 0, n, true)) return st;
    if (n > 0) {
        if (sphmp_status st = unpack_field_staged(dst, SPHMP_F_ALPHA, xa, n)) return st;
        if (sphmp_status st = unpack_field_staged(dst, SPHMP_F_APREV, xg, n)) return st;
    }
    return SPHMP_OK;
}

sphmp_status sphmp_compare_states(sphmp_ctx* a, sphmp_ctx* b, double* out, int32_t nout) {
    if (!a || !b || !out) return fail(SPHMP_ERR_INVALID_ARG, "bad arguments");
    if (nout < 5) return fail(SPHMP_ERR_INVALID_ARG, "need 5 output slots");
    if (a == b || a->device != b->device) return fail(SPHMP_ERR_INVALID_ARG, "need two contexts on one device");
    if (sphmp_status st = refresh_n(a)) return st;
    if (sphmp_status st = refresh_n(b)) return st;
    const int msize = a->cap > b->cap ? a->cap : b->cap;
    if (b->cmap_size < msize) {
        cudaFree(b->cmap);
        b->cmap = nullptr;
        CK(cudaMalloc(&b->cmap, sizeof(int32_t) * (size_t)(msize > 0 ? msize : 1)));
        b->cmap_size = msize;
    }
    if (!b->cred) CK(cudaMalloc(&b->cred, sizeof(double) * 7));
    CK(cudaStreamSynchronize(a->stream));
    launch_compare(dev_params(a), a->B, a->cur, dev_params(b), b->B, b->cur, b->cmap, msize, b->cred, b->stream);
    CHECK_LAUNCH("compare states");
    double r[7];
    CK(cudaMemcpyAsync(r, b->cred, sizeof(r), cudaMemcpyDeviceToHost, b->stream));
    CK(cudaStreamSynchronize(b->stream));
    const double m = r[4] > 0 ? r[4] : 1.0;
    out[0] = sqrt(r[0] / m);
    out[1] = r[6];
    out[2] = sqrt(r[1] / m);
    out[3] = r[3] > 0 ? sqrt(r[2] / r[3]) : 0.0;
    out[4] = r[4];
    if (nout > 5) out[5] = sqrt(r[5] / m);
    return SPHMP_OK;
}

// Device-side clone between contexts of the same capacity, grid and phase count
// (the audit's copies): every array a step or a per-pass call reads, and the
// host-side state, so that dst continues exactly as src would. Neighbour lists
// are not copied (dst rebuilds them). Other contexts take sphmp_copy_state.
static sphmp_status clone_state(sphmp_ctx* dst, sphmp_ctx* src) {
    if (dst->cap != src->cap || dst->gcap != src->gcap || dst->prm.nphase != src->prm.nphase ||
        dst->device != src->device || dst->prm.gridtotal != src->prm.gridtotal)
        return sphmp_copy_state(dst, src);
    if (sphmp_status st = refresh_n(src)) return st;
    CK(cudaStreamSynchronize(src->stream));
    CK(cudaStreamSynchronize(dst->stream));
    const size_t N = (size_t)src->cap, G = (size_t)src->gcap;
    const cudaStream_t s = dst->stream;
    const DevBuffers& a = src->B;
    DevBuffers& b = dst->B;
    auto cp = [&](void* d, const void* x, size_t bytes) {
        return cudaMemcpyAsync(d, x, bytes, cudaMemcpyDeviceToDevice, s);
    };
    for (int f = 0; f < kNumFloat4Fields; f++)
        for (int k = 0; k < 2; k++) CK(cp(b.f4[f][k], a.f4[f][k], sizeof(float4) * N));
    CK(cp(b.densp, a.densp, sizeof(float2) * N));
    CK(cp(b.accel4, a.accel4, sizeof(float4) * N));
    CK(cp(b.drift4, a.drift4, sizeof(float4) * 3 * N));
    CK(cp(b.velxcor, a.velxcor, sizeof(float4) * N));
    CK(cp(b.pmod, a.pmod, sizeof(float) * N));
    CK(cp(b.mgcell, a.mgcell, sizeof(uint32_t) * N));
    CK(cp(b.midsort, a.midsort, sizeof(uint32_t) * N));
    CK(cp(b.mgndx, a.mgndx, sizeof(uint32_t) * N));
    CK(cp(b.mgridoff, a.mgridoff, sizeof(int32_t) * G));
    CK(cp(b.mgridcnt, a.mgridcnt, sizeof(int32_t) * G));
    CK(cp(b.key, a.key, sizeof(uint32_t) * N));
    CK(cp(b.octk, a.octk, sizeof(uint8_t) * N));
    CK(cp(b.ccount, a.ccount, sizeof(uint32_t) * (G + 1)));
    CK(cp(b.cstart, a.cstart, sizeof(uint32_t) * (G + 2)));
    CK(cp(b.cend, a.cend, sizeof(uint32_t) * G));
    CK(cp(b.opos, a.opos, sizeof(uint32_t) * N));
    CK(cp(b.oidx, a.oidx, sizeof(uint32_t) * N));
    CK(cp(b.osrc, a.osrc, sizeof(uint32_t) * N));
    CK(cp(b.oct_start, a.oct_start, sizeof(uint32_t) * 8 * G));
    CK(cp(b.act, a.act, sizeof(uint32_t) * G));
    CK(cp(b.act_n, a.act_n, sizeof(uint32_t)));
    CK(cp(b.nact, a.nact, sizeof(int32_t)));
    CK(cp(b.frame, a.frame, sizeof(int32_t)));
    CK(cp(b.color, a.color, sizeof(float4) * N));
    CK(cp(b.bornid, a.bornid, sizeof(int32_t) * N));
    CK(cp(b.mass_raw, a.mass_raw, sizeof(float) * N));
    CK(cudaMemsetAsync(b.err, 0, sizeof(uint32_t), s));
    CK(cudaStreamSynchronize(s));
    dst->n = src->n;
    dst->prm.num = src->prm.num;
    memcpy(dst->cur, src->cur, sizeof(dst->cur));
    dst->alpha_advanced = src->alpha_advanced;
    dst->grid_valid = src->grid_valid;
    dst->oct_valid = src->oct_valid;
    dst->oct_built = src->oct_built;
    dst->pos_sorted = src->pos_sorted;
    dst->hash_n = src->hash_n;
    dst->list_mode = src->list_mode;
    dst->nbr_valid = false;
    dst->n_stale = false;
    dst->emit_on = src->emit_on;
    dst->emitter = src->emitter;
    drop_graph(dst);  // a captured graph holds the old buffer selectors
    return SPHMP_OK;
}

// The stored densities recomputed at the current positions (sort, then the
// density pass: after a sort it takes the bucket kernel, several times faster
// than the cell search on the step's stale cell lists).
static sphmp_status recompute_density(sphmp_ctx* c) {
    if (sphmp_status st = sphmp_get_particle_index(c)) return st;
    if (sphmp_status st = sphmp_get_grid_list(c)) return st;
    if (sphmp_status st = sphmp_rearrange_data(c)) return st;
    return sphmp_compute_pressure(c);
}

sphmp_status sphmp_rollout(sphmp_ctx* c, sphmp_ctx* audit, sphmp_corrector* cor, int32_t factor, int32_t steps,
                           int32_t audit_every, double tol, sphmp_rollout_stats* stats) {
    if (!c || !audit || c == audit) return fail(SPHMP_ERR_INVALID_ARG, "need the context and a separate audit context");
    if (factor < 1 || steps < 0 || audit_every < 1 || !(tol > 0.0))
        return fail(SPHMP_ERR_INVALID_ARG, "factor >= 1, steps >= 0, audit_every >= 1 and tol > 0 required");
    struct ClearFresh {  // the skip never outlives the rollout, whichever way it returns
        sphmp_ctx* c;
        ~ClearFresh() { c->sorted_dens_fresh = false; }
    } clear_fresh{c};
    sphmp_rollout_stats S;
    memset(&S, 0, sizeof(S));
    int done = 0, plain_left = 0;
    int since = audit_every - 1;  // the first large step is audited
    while (done < steps) {
        if (plain_left > 0 || steps - done < factor) {
            const int k = plain_left > 0 ? (plain_left < steps - done ? plain_left : steps - done) : steps - done;
            if (sphmp_status st = sphmp_step(c, k, SPHMP_SCHEDULE_FUSED, 1)) return st;
            done += k;
            S.plain_steps += k;
            plain_left = plain_left > k ? plain_left - k : 0;
            continue;
        }
        if (++since >= audit_every) {
            since = 0;
            S.audits++;
            if (sphmp_status st = clone_state(audit, c)) return st;
            if (sphmp_status st = sphmp_step(audit, factor, SPHMP_SCHEDULE_FUSED, 0)) return st;
            if (sphmp_status st = sphmp_step_large(c, cor, factor, 1)) return st;
            if (sphmp_status st = recompute_density(c)) return st;
            if (sphmp_status st = recompute_density(audit)) return st;
            double e[5];
            if (sphmp_status st = sphmp_compare_states(audit, c, e, 5)) return st;
            if (e[0] > S.density_err_max) S.density_err_max = e[0];
            if (e[2] > S.alpha_err_max) S.alpha_err_max = e[2];
            if (!(e[0] <= tol && e[2] <= tol)) {  // NaN counts as a failure
                S.fallbacks++;
                if (sphmp_status st = clone_state(c, audit)) return st;
                S.plain_steps += factor;
                plain_left = audit_every * factor;
                since = audit_every - 1;  // the first large step after the plain window is audited
            } else {
                S.large_steps++;
                c->sorted_dens_fresh = true;  // the next large step starts from this sort and density pass
            }
        } else {
            if (sphmp_status st = sphmp_step_large(c, cor, factor, 1)) return st;
            S.large_steps++;
        }
        done += factor;
    }
    CK(cudaStreamSynchronize(c->stream));
    if (stats) *stats = S;
    return take_device_errors(c, nullptr);
}

sphmp_status sphmp_conservation(sphmp_ctx* c, double* out, int32_t nout) {
    if (sphmp_status st = need_ctx(c)) return st;
    if (!out || nout < 3 + c->prm.nphase) return fail(SPHMP_ERR_INVALID_ARG, "need %d output slots", 3 + c->prm.nphase);
    const DevParams P = dev_params(c);
    launch_conservation(P, c->B, c->cur, c->stream);
    CHECK_LAUNCH("conservation");
    double red[16];
    CK(cudaMemcpyAsync(red, c->B.red, sizeof(red), cudaMemcpyDeviceToHost, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    out[0] = red[0];
    out[1] = red[1];
    for (int k = 0; k < c->prm.nphase; k++) out[2 + k] = red[2 + k];
    out[2 + c->prm.nphase] = red[5];
    return SPHMP_OK;
}

// ===========================================================================
// Reference entry-point names over a default context
// ===========================================================================

static sphmp_ctx* g_legacy = nullptr;
static std::mutex g_legacy_mu;

static void legacy_report(const char* call, sphmp_status st) {
    if (st != SPHMP_OK) fprintf(stderr, "CUDA ERROR: %s: %s\n", call, g_err.c_str());
}

static void legacy_run(const char* call, sphmp_status (*fn)(sphmp_ctx*)) {
    std::lock_guard<std::mutex> lk(g_legacy_mu);
    if (!g_legacy) {
        fail(SPHMP_ERR_STATE, "FluidSetupCUDA has not been called");
        legacy_report(call, SPHMP_ERR_STATE);
        return;
    }
    sphmp_status st = fn(g_legacy);
    if (st == SPHMP_OK) st = sphmp_sync(g_legacy);
    legacy_report(call, st);
}

// PressureSolve's stopping rule for the reference-named call (the reference's own
// loop has its break commented out and never returns): mean |density residue|
// over in-grid fluid particles at most 0.1 kg/m^3 after at least 2 iterations,
// the residue threshold and minimum of the reference's commented criterion
// (fluid_system_host.cu:543-546), and at most 100 iterations.
static sphmp_status legacy_pressure_solve(sphmp_ctx* c) {
    return sphmp_iisph_pressure_solve(c, 0.1f, 2, 100, nullptr, nullptr);
}

sphmp_ctx* sphmp_legacy_context(void) { return g_legacy; }

void cudaInit(int, char**) {
    cudaDeviceProp p;
    if (cudaGetDeviceProperties(&p, 0) != cudaSuccess) {
        fprintf(stderr, "CUDA ERROR: cudaInit: no device\n");
        return;
    }
    printf("-- CUDA --\n");
    printf("Name:       %s\n", p.name);
    printf("Revision:   %d.%d\n", p.major, p.minor);
    printf("Global Mem: %zu\n", p.totalGlobalMem);
    printf("Shared/Blk: %zu\n", p.sharedMemPerBlock);
    printf("Regs/Blk:   %d\n", p.regsPerBlock);
    printf("Warp Size:  %d\n", p.warpSize);
    printf("Thrds/Blk:  %d\n", p.maxThreadsPerBlock);
    printf("SMs:        %d\n", p.multiProcessorCount);
}

void cudaExit(int, char**) {}

void FluidClearCUDA(void) {
    std::lock_guard<std::mutex> lk(g_legacy_mu);
    sphmp_destroy(g_legacy);
    g_legacy = nullptr;
}

void FluidSetupCUDA(const sphmp_params* params) {
    std::lock_guard<std::mutex> lk(g_legacy_mu);
    if (!params) {
        fail(SPHMP_ERR_INVALID_ARG, "params is NULL");
        legacy_report("FluidSetupCUDA", SPHMP_ERR_INVALID_ARG);
        return;
    }
    sphmp_params p;
    sphmp_params_default(&p);
    memcpy(&p, params, 464);  // the ParamCarrier prefix
    p.nphase = SPHMP_MAX_PHASES;
    sphmp_destroy(g_legacy);
    g_legacy = nullptr;
    legacy_report("FluidSetupCUDA", sphmp_create(&p, &g_legacy));
}

void GetParticleIndexCUDA(void) { legacy_run("InsertParticlesCUDA", sphmp_get_particle_index); }
void GetGridListCUDA(void) { legacy_run("Sort Grid", sphmp_get_grid_list); }
void RearrageDataCUDA(void) { legacy_run("Sorting Failed", sphmp_rearrange_data); }
void InitialSortCUDA(uint32_t*, uint32_t*, int*) { GetParticleIndexCUDA(); }
void SortGridCUDA(int*) { GetGridListCUDA(); }
void CountingSortFullCUDA_(uint32_t*) { RearrageDataCUDA(); }
void MfComputePressureCUDA(void) { legacy_run("MfComputePressureCUDA", sphmp_compute_pressure); }
void MfComputeDriftVelCUDA(void) { legacy_run("MfComputeDriftVelCUDA", sphmp_compute_drift_vel); }
void MfComputeAlphaAdvanceCUDA(void) { legacy_run("MfComputeAlphaAdvanceCUDA", sphmp_compute_alpha_advance); }
void MfComputeCorrectionCUDA(void) { legacy_run("MfComputeCorrectionCUDA", sphmp_compute_correction); }
void MfComputeForceCUDA(void) { legacy_run("MfComputeForceCUDA", sphmp_compute_force); }
void ComputeForceCUDA_ProjectU(void) { legacy_run("MfComputeForceCUDA", sphmp_compute_force_projectu); }
void MfAdvanceCUDA(void) { legacy_run("MfAdvanceCUDA", sphmp_advance); }
void ComputeBoundaryDensity(void) { legacy_run("ComputeBoundaryDensity", sphmp_compute_boundary_density); }
void ComputeDensityIISPH_CUDA(void) { legacy_run("ComputeDensityIISPH_CUDA", sphmp_iisph_density); }
void PredictAdvection(void) { legacy_run("PredictAdvection", sphmp_iisph_predict_advection); }
void PressureSolve(void) { legacy_run("PressureSolve", legacy_pressure_solve); }
void Integration(void) { legacy_run("Integration", sphmp_iisph_integrate); }

void computeNumBlocks(int numPnts, int maxThreads, int* numBlocks, int* numThreads) {
    int t = numPnts < maxThreads ? numPnts : maxThreads;
    int b;
    if (t == 0) b = 1;
    else b = (numPnts % t != 0) ? (numPnts / t + 1) : (numPnts / t);
    if (t == 0) t = 1;
    if (numBlocks) *numBlocks = b;
    if (numThreads) *numThreads = t;
}

void TransferToCUDA(const sphmp_display_pack* disp, const sphmp_calc_pack* calc, int n) {
    std::lock_guard<std::mutex> lk(g_legacy_mu);
    sphmp_status st = g_legacy ? sphmp_upload_aos(g_legacy, disp, calc, n)
                               : fail(SPHMP_ERR_STATE, "FluidSetupCUDA has not been called");
    legacy_report("TransferToCUDA", st);
}

void TransferFromCUDA(sphmp_display_pack* disp, int n) {
    std::lock_guard<std::mutex> lk(g_legacy_mu);
    sphmp_status st = g_legacy ? sphmp_download_aos(g_legacy, disp, nullptr, n)
                               : fail(SPHMP_ERR_STATE, "FluidSetupCUDA has not been called");
    legacy_report("TransferFromCUDA", st);
}

void EmitUpdateCUDA(int startnum, int endnum, const sphmp_display_pack* disp, const sphmp_calc_pack* calc) {
    std::lock_guard<std::mutex> lk(g_legacy_mu);
    sphmp_status st = g_legacy ? sphmp_emit_aos(g_legacy, disp ? disp + startnum : nullptr,
                                                calc ? calc + startnum : nullptr, startnum, endnum)
                               : fail(SPHMP_ERR_STATE, "FluidSetupCUDA has not been called");
    legacy_report("EmitUpdateCUDA", st);
}

}  // extern "C"

// CarryParam(ParamCarrier&) with the reference's C++ linkage.
struct ParamCarrier;
void CarryParam(ParamCarrier& hostCarrier) {
    std::lock_guard<std::mutex> lk(g_legacy_mu);
    if (!g_legacy) {
        fail(SPHMP_ERR_STATE, "FluidSetupCUDA has not been called");
        legacy_report("CarryParam", SPHMP_ERR_STATE);
        return;
    }
    sphmp_params p = g_legacy->prm;
    memcpy(&p, &hostCarrier, 464);
    legacy_report("CarryParam", sphmp_set_params(g_legacy, &p));
}
