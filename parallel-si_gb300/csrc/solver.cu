// solver.cu -- host orchestration of one solver: device memory, the
// evaluation pipeline, the switch step and the solve_si loop.
#include <algorithm>
#include <cstring>
#include <string>

#include "device_common.cuh"
#include "kernels.h"
#include "psi_internal.h"
#include "solver.h"

namespace psi {

namespace {

int ceil_log2(int64_t x)
{
    int r = 0;
    while (((int64_t)1 << r) < x) r++;
    return r;
}

}  // namespace

int Solver::set_device()
{
    PSI_CUDA_TRY(cudaSetDevice(device_));
    return PSI_OK;
}

namespace {

int check_options(const psi_options &opt)
{
    if (opt.valuation_mode != PSI_VAL_PATH) return fail(PSI_ERR_INVALID, "unknown valuation_mode");
    if (opt.sublist_len < 2) return fail(PSI_ERR_INVALID, "sublist_len must be >= 2");
    if (opt.incremental < PSI_INCR_OFF || opt.incremental > PSI_INCR_ALWAYS)
        return fail(PSI_ERR_INVALID, "unknown incremental mode");
    if (opt.patch_limit < 0) return fail(PSI_ERR_INVALID, "patch_limit must be >= 0");
    if (opt.walk_block != 0 && (opt.walk_block < 32 || opt.walk_block > 1024 || opt.walk_block % 32 != 0))
        return fail(PSI_ERR_INVALID, "walk_block must be 0 or a multiple of 32 in [32, 1024]");
    if (opt.switch_kernel != PSI_SWITCH_THREAD && opt.switch_kernel != PSI_SWITCH_WARP)
        return fail(PSI_ERR_INVALID, "unknown switch_kernel");
    int ndev = 0;
    cudaError_t e = cudaGetDeviceCount(&ndev);
    if (e != cudaSuccess || ndev == 0) return fail(PSI_ERR_NO_DEVICE, "no CUDA device available");
    if (opt.device < 0 || opt.device >= ndev) return fail(PSI_ERR_INVALID, "device ordinal out of range");
    return PSI_OK;
}

}  // namespace

int Solver::create(const CsrView &g, const psi_options &opt, Solver **out, bool validate)
{
    *out = nullptr;
    if (g.n < 0) return fail(PSI_ERR_INVALID, "negative vertex count");   // n = 0: the empty game
    if (2 * (int64_t)g.n + 2 > INT32_MAX) return fail(PSI_ERR_TOO_LARGE, "n too large for int32 tour ids");
    int rc = check_options(opt);
    if (rc) return rc;
    Solver *s = new Solver();
    s->device_ = opt.device;
    s->timing_ = opt.timing != 0;
    s->stride_ = opt.sublist_len;
    s->use_graph_ = opt.graph != 0;
    s->incremental_ = opt.incremental;
    s->patch_limit_ = opt.patch_limit;
    s->walk_block_ = opt.walk_block ? opt.walk_block : kWalkBlock;
    s->switch_warp_ = opt.switch_kernel == PSI_SWITCH_WARP;
    rc = s->alloc_arrays(g.n, g.m);
    if (!rc) rc = s->upload_game(g, validate);
    if (rc) {
        delete s;
        return rc;
    }
    *out = s;
    return PSI_OK;
}

int Solver::create_arena(int64_t max_vertices, int64_t max_edges, int32_t slots, const psi_options &opt,
                         Solver **out)
{
    *out = nullptr;
    if (max_vertices < 2 || max_edges < 1 || slots < 1) return fail(PSI_ERR_INVALID, "empty arena");
    if (2 * max_vertices + 2 > INT32_MAX || max_edges > INT32_MAX)
        return fail(PSI_ERR_TOO_LARGE, "arena too large for int32 ids");
    int rc = check_options(opt);
    if (rc) return rc;
    Solver *s = new Solver();
    s->device_ = opt.device;
    s->timing_ = opt.timing != 0;
    s->stride_ = opt.sublist_len;
    // admissions list their new vertices as changed ones: a patch evaluates them
    s->incremental_ = opt.incremental;
    s->patch_limit_ = opt.patch_limit;
    s->walk_block_ = opt.walk_block ? opt.walk_block : kWalkBlock;
    s->switch_warp_ = opt.switch_kernel == PSI_SWITCH_WARP;
    rc = s->alloc_arrays(max_vertices, max_edges);
    if (!rc) rc = s->init_arena(slots);
    if (rc) {
        delete s;
        return rc;
    }
    *out = s;
    return PSI_OK;
}

// Many games as one disjoint union (a batch): each game's arrays are copied
// as they are to their place in the device union and shifted there (no host
// packing); base receives the first vertex of every game (K+1 entries).
int Solver::create_union(const std::vector<const HostGame *> &gs, const psi_options &opt, Solver **out,
                         std::vector<int64_t> *base)
{
    *out = nullptr;
    const int32_t K = (int32_t)gs.size();
    if (K < 1) return fail(PSI_ERR_INVALID, "empty batch");
    std::vector<int32_t> table(2 * (size_t)K + 2);
    int32_t *ub = table.data(), *ue = ub + K + 1;
    int64_t n = 0, m = 0;
    int32_t top = 0;
    base->assign(1, 0);
    for (int32_t k = 0; k < K; k++) {
        const HostGame *g = gs[k];
        if (!g || g->n <= 0) return fail(PSI_ERR_INVALID, "empty game in batch");
        ub[k] = (int32_t)n;
        ue[k] = (int32_t)m;
        n += g->n;
        m += g->m;
        top = g->max_pri > top ? g->max_pri : top;
        base->push_back(n);
        if (2 * n + 2 > INT32_MAX) return fail(PSI_ERR_TOO_LARGE, "batch has too many vertices for int32 tour ids");
        if (m > INT32_MAX) return fail(PSI_ERR_TOO_LARGE, "batch has more than 2^31-1 edges");
    }
    ub[K] = (int32_t)n;
    ue[K] = (int32_t)m;
    int rc = check_options(opt);
    if (rc) return rc;
    Solver *s = new Solver();
    s->device_ = opt.device;
    s->timing_ = opt.timing != 0;
    s->stride_ = opt.sublist_len;
    s->use_graph_ = opt.graph != 0;
    s->incremental_ = opt.incremental;
    s->patch_limit_ = opt.patch_limit;
    s->walk_block_ = opt.walk_block ? opt.walk_block : kWalkBlock;
    s->switch_warp_ = opt.switch_kernel == PSI_SWITCH_WARP;
    rc = s->alloc_arrays(n, m);
    if (!rc) rc = s->upload_union(gs, table, base->back());
    if (rc) {
        delete s;
        return rc;
    }
    s->max_pri_ = top;
    *out = s;
    return PSI_OK;
}

int Solver::upload_union(const std::vector<const HostGame *> &gs, const std::vector<int32_t> &table, int64_t n)
{
    const int32_t K = (int32_t)gs.size();
    const int32_t *ub = table.data(), *ue = ub + K + 1;
    set_extent((int32_t)n);
    m_ = ue[K];
    np_ = n_;
    const struct {
        void **ptr;
        size_t bytes;
    } arrays[] = {{(void **)&game_of_, 4 * (size_t)n_}, {(void **)&gstate_, sizeof(int4) * (size_t)K},
                  {(void **)&gcount_, sizeof(unsigned long long) * (size_t)K}};
    for (const auto &a : arrays) {
        cudaError_t e = device_alloc(a.ptr, a.bytes, stream_);
        if (e != cudaSuccess) return fail(PSI_ERR_NOMEM, std::string("device allocation: ") + cudaGetErrorString(e));
        allocs_.push_back(*a.ptr);
    }
    int32_t *d_tab = nullptr;
    PSI_CUDA_TRY(device_alloc((void **)&d_tab, 4 * table.size(), stream_));
    PSI_CUDA_TRY(cudaMemcpyAsync(d_tab, table.data(), 4 * table.size(), cudaMemcpyHostToDevice, stream_));
    for (int32_t k = 0; k < K; k++) {
        const HostGame &g = *gs[k];
        const size_t nb = 4 * (size_t)g.n;
        PSI_CUDA_TRY(cudaMemcpyAsync(st_ + ub[k], g.owner.data(), nb, cudaMemcpyHostToDevice, stream_));
        PSI_CUDA_TRY(cudaMemcpyAsync(pri_ + ub[k], g.priority.data(), nb, cudaMemcpyHostToDevice, stream_));
        PSI_CUDA_TRY(cudaMemcpyAsync(off_ + ub[k], g.offsets.data(), nb, cudaMemcpyHostToDevice, stream_));
        if (g.m)
            PSI_CUDA_TRY(cudaMemcpyAsync(tgt_ + ue[k], g.targets.data(), 4 * (size_t)g.m, cudaMemcpyHostToDevice,
                                         stream_));
    }
    launch_union_fixup(stream_, n_, m_, K, d_tab, d_tab + K + 1, off_, tgt_, game_of_);
    PSI_CUDA_TRY(cudaMemsetAsync(gcount_, 0, 8 * (size_t)K, stream_));
    cudaFreeAsync(d_tab, stream_);
    games_ = K;
    return finish_upload();
}

// Vertex count the kernels process: the tour has 2n+2 nodes, the sublist
// heads follow from the stride.
void Solver::set_extent(int32_t n)
{
    n_ = n;
    L_ = 2 * (int64_t)n_ + 2;
    // heads at node j*stride for j < nsub-1, plus the list start (node L-1)
    nsub_ = (int32_t)(ceil_div(L_ - 1, stride_) + 1);
}

// Device arrays for games of up to cap_n vertices and cap_m edges.
int Solver::alloc_arrays(int64_t cap_n, int64_t cap_m)
{
    int rc = set_device();
    if (rc) return rc;
    cap_n_ = cap_n;
    cap_m_ = cap_m;
    const int64_t capL = 2 * cap_n + 2;
    const int64_t cap_sub = ceil_div(capL - 1, stride_) + 1;
    // incremental evaluation: change-list capacity (larger lists mean a full
    // evaluation), re-evaluated set capacity, level cap of its search
    if (incremental_ != PSI_INCR_OFF) {
        const bool always = incremental_ == PSI_INCR_ALWAYS;
        const int64_t cc = always ? cap_n : patch_limit_ > 0 ? patch_limit_ : std::max<int64_t>(1024, cap_n >> 6);
        const int64_t ac = always ? cap_n : std::max<int64_t>(4096, cap_n >> 3);
        ccap_ = (int32_t)std::max<int64_t>(1, std::min(cc, cap_n));
        acap_ = (int32_t)std::max<int64_t>(1, std::min(ac, cap_n));
        max_levels_ = always ? INT32_MAX : 256;
    }
    ucap_ = cap_n + acap_;
    PSI_CUDA_TRY(cudaStreamCreateWithFlags(&stream_, cudaStreamNonBlocking));
    for (auto &p : ph_) {
        PSI_CUDA_TRY(cudaEventCreate(&p.a));
        PSI_CUDA_TRY(cudaEventCreate(&p.b));
    }
    PSI_CUDA_TRY(cudaEventCreate(&region_a_));
    PSI_CUDA_TRY(cudaEventCreate(&region_b_));
    const struct {
        void **ptr;
        size_t bytes;
    } arrays[] = {
        {(void **)&owner_, (size_t)cap_n},
        {(void **)&pri_, 4 * (size_t)cap_n},
        {(void **)&off_, 4 * ((size_t)cap_n + 1)},
        {(void **)&tgt_, 4 * (size_t)cap_m},
        {(void **)&rev_off_, 4 * ((size_t)cap_n + 1)},
        {(void **)&rev_src_, 4 * (size_t)cap_m},
        {(void **)&plist_, 4 * (size_t)cap_n},
        {(void **)&strat_, 4 * (size_t)cap_n},
        {(void **)&st_, 4 * (size_t)cap_n},
        {(void **)&solved_, (size_t)cap_n},
        {(void **)&node_, sizeof(PathNode) * (size_t)cap_n},
        {(void **)&skip_, sizeof(int4) * (size_t)cap_n},
        {(void **)&key_, 4 * (size_t)cap_n},
        {(void **)&succ_, 4 * (size_t)capL},
        {(void **)&dirty_, (size_t)cap_n},
        {(void **)&need_, (size_t)cap_n},
        {(void **)&tie_, (size_t)cap_n},
        {(void **)&watch_, (size_t)cap_n},
        {(void **)&ulist_, 4 * (size_t)ucap_},
        {(void **)&vloc_, 8 * (size_t)cap_n},
        {(void **)&redA_, 8 * (size_t)cap_sub},
        {(void **)&redB_, 8 * (size_t)cap_sub},
        {(void **)&redC_, 8 * (size_t)cap_sub},
        {(void **)&jA_, sizeof(int4) * (size_t)cap_n},
        {(void **)&jB_, sizeof(int4) * (size_t)cap_n},
        {(void **)&dw_, sizeof(Words)},
        {(void **)&ctl_, sizeof(GraphCtl)},
    };
    for (const auto &a : arrays) {
        cudaError_t e = device_alloc(a.ptr, a.bytes, stream_);
        if (e != cudaSuccess) return fail(PSI_ERR_NOMEM, std::string("device allocation: ") + cudaGetErrorString(e));
        allocs_.push_back(*a.ptr);
    }
    if (incremental_ != PSI_INCR_OFF) {
        const struct {
            void **ptr;
            size_t bytes;
        } patch[] = {
            {(void **)&clist_, 4 * (size_t)ccap_},
            {(void **)&alist_, 4 * (size_t)acap_},
            {(void **)&apos_, 4 * (size_t)std::max<int64_t>(1, cap_n)},
            {(void **)&pj_, (3 * sizeof(int4) + sizeof(int2)) * (size_t)acap_},
        };
        for (const auto &a : patch) {
            cudaError_t e = device_alloc(a.ptr, a.bytes, stream_);
            if (e != cudaSuccess)
                return fail(PSI_ERR_NOMEM, std::string("device allocation: ") + cudaGetErrorString(e));
            allocs_.push_back(*a.ptr);
        }
        PSI_CUDA_TRY(cudaMemsetAsync(apos_, 0xff, 4 * (size_t)std::max<int64_t>(1, cap_n), stream_));   // -1: in no patch
    }
    PSI_CUDA_TRY(cudaMallocHost((void **)&hw_, sizeof(Words)));
    PSI_CUDA_TRY(cudaMemsetAsync(dw_, 0, sizeof(Words), stream_));
    const GraphCtl fresh;
    // pageable source: staged before the call returns
    PSI_CUDA_TRY(cudaMemcpyAsync(ctl_, &fresh, sizeof fresh, cudaMemcpyHostToDevice, stream_));
    PSI_CUDA_TRY(cudaMemsetAsync(dirty_, 0, (size_t)cap_n, stream_));
    return PSI_OK;
}

// One game filling the arrays: upload, player lists, reverse CSR.  The
// owner array goes up as the caller's int32 (into st_, free until the first
// evaluation) and is narrowed on the device; the player lists are an ordered
// partition on the device.
int Solver::upload_game(const CsrView &g, bool validate)
{
    set_extent(g.n);
    m_ = g.m;
    max_pri_ = g.max_pri;
    np_ = n_;
    PSI_CUDA_TRY(cudaMemcpyAsync(st_, g.owner, 4 * (size_t)n_, cudaMemcpyHostToDevice, stream_));
    PSI_CUDA_TRY(cudaMemcpyAsync(pri_, g.priority, 4 * (size_t)n_, cudaMemcpyHostToDevice, stream_));
    PSI_CUDA_TRY(cudaMemcpyAsync(off_, g.offsets, 4 * ((size_t)n_ + 1), cudaMemcpyHostToDevice, stream_));
    if (m_) PSI_CUDA_TRY(cudaMemcpyAsync(tgt_, g.targets, 4 * (size_t)m_, cudaMemcpyHostToDevice, stream_));
    if (validate) {
        int64_t bad_v = -1;
        int32_t check = 0, bad_e = 0, top = 0;
        int ve = validate_game(stream_, n_, m_, st_, pri_, off_, tgt_, &bad_v, &check, &bad_e, &top);
        if (ve) return fail(PSI_ERR_CUDA, std::string("validation: ") + cudaGetErrorString((cudaError_t)ve));
        if (bad_v >= 0) {
            std::string v = std::to_string(bad_v);
            if (check == 1) return fail(PSI_ERR_INVALID, "invalid player at vertex " + v);
            if (check == 2) return fail(PSI_ERR_INVALID, "negative priority at vertex " + v);
            return fail(PSI_ERR_INVALID, "vertex " + v + " has no successor");
        }
        if (bad_e) return fail(PSI_ERR_INVALID, "successor out of range");
        max_pri_ = top;
    }
    return finish_upload();
}

// Common tail of an upload: the owner array (uploaded as int32 into st_)
// narrowed, the player lists, fresh SI state and the reverse CSR.
int Solver::finish_upload()
{
    launch_narrow_owner(stream_, n_, st_, owner_);
    int ce = partition_players(stream_, n_, owner_, plist_, &dw_->sinkcount);
    if (ce) return fail(PSI_ERR_CUDA, std::string("player lists: ") + cudaGetErrorString((cudaError_t)ce));
    PSI_CUDA_TRY(cudaMemsetAsync(solved_, 0, n_, stream_));
    PSI_CUDA_TRY(cudaMemsetAsync(st_, 0, 4 * (size_t)n_, stream_));
    reset_tracking();
    // reverse CSR on the device (distinct in-neighbours, increasing order)
    int64_t rev_m = 0;
    ce = build_reverse_csr(stream_, n_, m_, off_, tgt_, rev_off_, rev_src_, &rev_m);
    if (ce) return fail(PSI_ERR_CUDA, std::string("reverse CSR: ") + cudaGetErrorString((cudaError_t)ce));
    int rc = sync_and_check("upload");
    if (rc) return rc;
    np0_ = hw_->sinkcount;
    return PSI_OK;
}

Solver::~Solver()
{
    cudaSetDevice(device_);
    if (stream_) cudaStreamSynchronize(stream_);
    if (graph_exec_) cudaGraphExecDestroy(graph_exec_);
    if (graph_) cudaGraphDestroy(graph_);
    for (void *p : allocs_) cudaFreeAsync(p, stream_);   // back to the library's pool
    if (stream_) cudaStreamSynchronize(stream_);
    if (hw_) cudaFreeHost(hw_);
    for (auto &p : ph_) {
        if (p.a) cudaEventDestroy(p.a);
        if (p.b) cudaEventDestroy(p.b);
    }
    if (region_a_) cudaEventDestroy(region_a_);
    if (region_b_) cudaEventDestroy(region_b_);
    if (stream_) cudaStreamDestroy(stream_);
}

int Solver::timer_begin()
{
    int rc = set_device();
    if (rc) return rc;
    PSI_CUDA_TRY(cudaStreamSynchronize(stream_));
    PSI_CUDA_TRY(cudaEventRecord(region_a_, stream_));
    return PSI_OK;
}

int Solver::timer_end(double *ms)
{
    int rc = set_device();
    if (rc) return rc;
    PSI_CUDA_TRY(cudaEventRecord(region_b_, stream_));
    PSI_CUDA_TRY(cudaEventSynchronize(region_b_));
    float f = 0;
    PSI_CUDA_TRY(cudaEventElapsedTime(&f, region_a_, region_b_));
    *ms = f;
    return PSI_OK;
}

void Solver::phase_begin(Phase p)
{
    if (timing_) cudaEventRecord(ph_[p].a, stream_);
}

void Solver::phase_end(Phase p)
{
    if (!timing_) return;
    cudaEventRecord(ph_[p].b, stream_);
    ph_[p].pending = true;
}

// Called after a stream synchronisation: adds the elapsed time of every phase
// recorded since the last collection.
int Solver::collect_phases()
{
    for (int i = 0; i < PH_COUNT; i++) {
        if (!ph_[i].pending) continue;
        float ms = 0;
        PSI_CUDA_TRY(cudaEventElapsedTime(&ms, ph_[i].a, ph_[i].b));
        times_.ms[i] += ms;
        times_.calls[i]++;
        ph_[i].pending = false;
    }
    return PSI_OK;
}

int Solver::sync_and_check(const char *what)
{
    PSI_CUDA_TRY(cudaGetLastError());
    PSI_CUDA_TRY(cudaMemcpyAsync(hw_, dw_, sizeof(Words), cudaMemcpyDeviceToHost, stream_));
    cudaError_t e = cudaStreamSynchronize(stream_);
    if (e != cudaSuccess) return fail(PSI_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
    int rc = collect_phases();
    if (rc) return rc;
    times_.patches = (int64_t)hw_->patch[0];
    times_.patched = (int64_t)hw_->patch[1];
    times_.tour_parents = (int64_t)hw_->relink[0];
    times_.tour_entries = (int64_t)hw_->relink[1];
    times_.tour_children = (int64_t)hw_->relink[2];
    if (hw_->err) {
        uint32_t bits = hw_->err;
        cudaMemsetAsync(dw_, 0, sizeof(Words), stream_);
        cudaStreamSynchronize(stream_);
        return fail(PSI_ERR_LIMIT, std::string(what) + ": device step cap reached (bits " + std::to_string(bits) + ")");
    }
    return PSI_OK;
}

void Solver::reset_times()
{
    times_ = SolverTimes();
    cudaMemsetAsync(dw_->patch, 0, sizeof(dw_->patch), stream_);
    cudaMemsetAsync(dw_->relink, 0, sizeof(dw_->relink), stream_);
    if (hw_) hw_->patch[0] = hw_->patch[1] = hw_->relink[0] = hw_->relink[1] = hw_->relink[2] = 0;
}

void Solver::reset_tracking()
{
    static const int32_t one = 1;
    cudaMemsetAsync(need_, 1, (size_t)n_, stream_);
    cudaMemsetAsync(tie_, 0, (size_t)n_, stream_);
    cudaMemsetAsync(watch_, 0, (size_t)n_, stream_);
    cudaMemcpyAsync(&ctl_->quiet, &one, sizeof one, cudaMemcpyHostToDevice, stream_);
}

int Solver::init_strat()
{
    int rc = set_device();
    if (rc) return rc;
    launch_init_strat(stream_, n_, owner_, off_, tgt_, strat_, st_);
    PSI_CUDA_TRY(cudaMemsetAsync(solved_, 0, n_, stream_));
    reset_tracking();
    rc = sync_and_check("init_strat");
    if (rc) return rc;
    strat_ready_ = true;
    val_ready_ = false;
    tour_valid_ = false;
    return PSI_OK;
}

int Solver::reset_opponent_strategy()
{
    if (!strat_ready_) return fail(PSI_ERR_STATE, "reset_opponent_strategy before init_strat");
    int rc = set_device();
    if (rc) return rc;
    launch_reset_odd(stream_, n_, owner_, off_, tgt_, strat_);
    reset_tracking();   // Odd's choices start over
    tour_valid_ = false;
    return sync_and_check("reset_opponent_strategy");
}

PatchArgs Solver::patch_args()
{
    PatchArgs a;
    a.g = ctl_;
    a.ucount = &dw_->ucount;
    a.sinkcount = &dw_->sinkcount;
    a.clist = clist_;
    a.strat = strat_;
    a.pri = pri_;
    a.rev_off = rev_off_;
    a.rev_src = rev_src_;
    a.solved = solved_;
    a.alist = alist_;
    a.apos = apos_;
    a.rel = pj_;
    a.sja = pj_ ? pj_ + acap_ : nullptr;
    a.sjb = pj_ ? pj_ + 2 * (size_t)acap_ : nullptr;
    a.arev = pj_ ? reinterpret_cast<int2 *>(pj_ + 3 * (size_t)acap_) : nullptr;
    a.acap = acap_;
    a.ccap = ccap_;
    a.max_levels = max_levels_;
    a.ucap = ucap_;
    a.st = st_;
    a.node = node_;
    a.key = key_;
    a.ulist = ulist_;
    a.stats = dw_->patch;
    a.track = track();
    a.skip = skip_;
    return a;
}

int Solver::enqueue_eval(bool timed)
{
    int rc = enqueue_patch(timed);
    if (!rc) rc = enqueue_full(timed);
    if (rc) return rc;
    PSI_CUDA_TRY(cudaMemsetAsync(&ctl_->quiet, 0, sizeof(int32_t), stream_));
    return PSI_OK;
}

// 0. a patch, when the gates allow it and it succeeds; otherwise its
//    kernels return at once and the full evaluation's gates are open
int Solver::enqueue_patch(bool timed)
{
    if (timed) phase_begin(PH_PATCH);
    const PatchArgs pa = patch_args();
    launch_patch_begin(stream_, pa);
    if (incremental_ != PSI_INCR_OFF) {
        int pe = launch_patch_collect(stream_, pa);
        if (!pe) pe = launch_patch_values(stream_, pa);
        if (pe) return fail(PSI_ERR_CUDA, std::string("patch kernels: ") + cudaGetErrorString((cudaError_t)pe));
    }
    if (timed) phase_end(PH_PATCH);
    return PSI_OK;
}

// The full evaluation, every kernel gated (ctl_->full / incr / eval).
int Solver::enqueue_full(bool timed)
{
    auto begin = [&](Phase p) {
        if (timed) phase_begin(p);
    };
    auto end = [&](Phase p) {
        if (timed) phase_end(p);
    };
    // 1. Euler tour of the sink tree: built afresh (gate full) or the previous
    //    one relinked where strategies or solved flags changed (gate incr);
    //    jA_ is free until the cycle pass: it holds the list of dirty parents
    begin(PH_TOUR);
    launch_tour_build(stream_, n_, strat_, solved_, rev_off_, rev_src_, succ_, vloc_, ulist_, &dw_->sinkcount, dirty_,
                      &ctl_->full, tie_, need_, dw_->relink);
    int ce = launch_tour_update(stream_, n_, strat_, solved_, rev_off_, rev_src_, dirty_, succ_, vloc_, ulist_,
                                &dw_->sinkcount, reinterpret_cast<int32_t *>(jA_), &dw_->cnt[0], &ctl_->incr, tie_,
                                need_, dw_->relink);
    if (ce) return fail(PSI_ERR_CUDA, std::string("tour update: ") + cudaGetErrorString((cudaError_t)ce));
    end(PH_TOUR);
    // 2. Helman-JaJa sublists, then the reduced list ranked on the device
    begin(PH_SUBLIST);
    launch_walk_sublists(stream_, nsub_, n_, L_, stride_, succ_, vloc_, redA_, &dw_->err, &ctl_->eval,
                         walk_block_);
    end(PH_SUBLIST);
    begin(PH_REDUCED);
    const int2 *fin = nullptr;
    ce = launch_rank_reduced(stream_, nsub_, redA_, redB_, redC_, &fin, &ctl_->eval, &dw_->err);
    if (ce) return fail(PSI_ERR_CUDA, std::string("reduced-list kernel: ") + cudaGetErrorString((cudaError_t)ce));
    end(PH_REDUCED);
    // 3. broadcast depths; collect the vertices the sink does not reach
    //    (ulist held the sink's children until here); root-path summaries
    begin(PH_BROADCAST);
    launch_broadcast_depth(stream_, n_, vloc_, fin, strat_, pri_, solved_, st_, node_, ulist_, &dw_->ucount,
                           &ctl_->eval);
    launch_rootinfo(stream_, n_, st_, node_, key_, &dw_->err, track(), &ctl_->eval, skip_);
    end(PH_BROADCAST);
    // 4. cycle parity by pointer jumping over the unreached vertices (the
    //    tour's vloc array is free again: it holds the two active lists)
    begin(PH_CYCLES);
    int32_t *la = reinterpret_cast<int32_t *>(vloc_), *lb = la + n_;
    ce = launch_cycles(stream_, &dw_->ucount, ulist_, strat_, pri_, solved_, st_, key_, jA_, jB_, la, lb, dw_->cnt,
                       &dw_->err, track(), &ctl_->eval);
    if (ce) return fail(PSI_ERR_CUDA, std::string("cycle kernel: ") + cudaGetErrorString((cudaError_t)ce));
    end(PH_CYCLES);
    return PSI_OK;
}

int Solver::compute_valuation()
{
    if (!strat_ready_) return fail(PSI_ERR_STATE, "compute_valuation before init_strat");
    int rc = set_device();
    if (rc) return rc;
    // the previous tour (and the switch steps' change list since) is usable
    // only if no strategy changed outside a switch step since it was built
    launch_eval_gates(stream_, ctl_, tour_valid_ ? 0 : 1, tour_valid_ ? 1 : 0,
                      (tour_valid_ && incremental_ != PSI_INCR_OFF) ? 1 : 0);
    const unsigned long long patches_before = hw_->patch[0];
    phase_begin(PH_EVAL);
    rc = enqueue_eval(true);
    if (rc) return rc;
    phase_end(PH_EVAL);
    rc = sync_and_check("compute_valuation");
    if (rc) return rc;
    if (hw_->patch[0] == patches_before) {   // a full evaluation: ucount is its unreached count
        int32_t nu = hw_->ucount;
        last_unreached_ = nu;
        times_.unreached += nu;
        if (nu > 0) times_.jump_rounds += ceil_log2(nu) + 1;
    }
    times_.evals++;
    val_ready_ = true;
    tour_valid_ = true;
    return PSI_OK;
}

int Solver::mark_solved(int32_t player)
{
    if (player != 0 && player != 1) return fail(PSI_ERR_INVALID, "player must be 0 or 1");
    if (!val_ready_) return fail(PSI_ERR_STATE, "mark_solved before compute_valuation");
    int rc = set_device();
    if (rc) return rc;
    // a masked step (served games) scans the whole list
    launch_mark_solved(stream_, &dw_->ucount, ulist_, player, st_, solved_, dirty_, gmask_ ? game_of_ : nullptr,
                       gmask_, nullptr, gmask_ ? nullptr : &ctl_->mfrom[player], &ctl_->mdone);
    PSI_CUDA_TRY(cudaGetLastError());
    return PSI_OK;   // ordered on the stream before the next call
}

int Solver::switch_strategy(int32_t player, int64_t *switched)
{
    if (player != 0 && player != 1) return fail(PSI_ERR_INVALID, "player must be 0 or 1");
    if (!val_ready_) return fail(PSI_ERR_STATE, "switch_strategy before compute_valuation");
    int rc = set_device();
    if (rc) return rc;
    PSI_CUDA_TRY(cudaMemsetAsync(dw_->sw, 0, sizeof(dw_->sw), stream_));
    phase_begin(PH_SWITCH);
    const int32_t np = (player == 0) ? np0_ : np_ - np0_;
    const int32_t *pl = plist_ + (player == 0 ? 0 : np0_);
    // jB_ is free until the next cycle pass: it holds the list of vertices to examine
    launch_switch(stream_, np, pl, player, off_, tgt_, strat_, st_, key_, node_, dw_->sw, game_of_, gcount_, gmask_,
                  dirty_, &dw_->err, nullptr, need_, reinterpret_cast<int32_t *>(jB_), &dw_->cnt[2], changes(), tie_,
                  watch_, skip_, switch_warp_, &dw_->claim, arena_ ? nullptr : owner_, n_);
    phase_end(PH_SWITCH);
    rc = sync_and_check("switch_strategy");
    if (rc) return rc;
    times_.switches++;
    times_.sw_edges += (int64_t)hw_->sw[0];
    times_.sw_loads += (int64_t)hw_->sw[1];
    times_.sw_changed += (int64_t)hw_->sw[2];
    if (switched) *switched = (int64_t)hw_->sw[3];
    return PSI_OK;
}

int Solver::get_infinite(int32_t *out)
{
    int rc = set_device();
    if (rc) return rc;
    std::vector<int32_t> st(n_);
    PSI_CUDA_TRY(cudaMemcpyAsync(st.data(), st_, 4 * (size_t)n_, cudaMemcpyDeviceToHost, stream_));
    PSI_CUDA_TRY(cudaStreamSynchronize(stream_));
    for (int32_t v = 0; v < n_; v++) out[v] = st_infinite(st[v]);
    return PSI_OK;
}

int Solver::get_depth(int32_t *out)
{
    int rc = set_device();
    if (rc) return rc;
    PSI_CUDA_TRY(cudaMemcpyAsync(out, st_, 4 * (size_t)n_, cudaMemcpyDeviceToHost, stream_));
    PSI_CUDA_TRY(cudaStreamSynchronize(stream_));
    return PSI_OK;
}

int Solver::get_winning(int32_t player, std::vector<int32_t> &out)
{
    int64_t k = 0;
    int rc = winning_ids(player, &k);
    if (rc) return rc;
    out.resize((size_t)k);
    return copy_winning(out.data(), k);
}

// The winning set of `player` selected on the device into succ_ (free between
// evaluations); *count receives its size.
int Solver::winning_ids(int32_t player, int64_t *count)
{
    if (player != 0 && player != 1) return fail(PSI_ERR_INVALID, "player must be 0 or 1");
    int rc = set_device();
    if (rc) return rc;
    int ce = select_winning(stream_, n_, player, st_, succ_, &dw_->sinkcount);
    if (ce) return fail(PSI_ERR_CUDA, std::string("winning set: ") + cudaGetErrorString((cudaError_t)ce));
    rc = sync_and_check("get_winning");
    if (rc) return rc;
    *count = hw_->sinkcount;
    return PSI_OK;
}

int Solver::copy_winning(int32_t *out, int64_t k)
{
    if (k > 0) PSI_CUDA_TRY(cudaMemcpyAsync(out, succ_, 4 * (size_t)k, cudaMemcpyDeviceToHost, stream_));
    PSI_CUDA_TRY(cudaStreamSynchronize(stream_));
    return PSI_OK;
}

int Solver::get_range(const int32_t *src, int64_t v0, int64_t count, int32_t *out)
{
    if (v0 < 0 || count < 0 || v0 + count > n_) return fail(PSI_ERR_INVALID, "vertex range out of bounds");
    int rc = set_device();
    if (rc) return rc;
    if (count) PSI_CUDA_TRY(cudaMemcpyAsync(out, src + v0, 4 * (size_t)count, cudaMemcpyDeviceToHost, stream_));
    PSI_CUDA_TRY(cudaStreamSynchronize(stream_));
    return PSI_OK;
}

int Solver::get_strategy_range(int64_t v0, int64_t count, int32_t *out) { return get_range(strat_, v0, count, out); }

int Solver::get_infinite_range(int64_t v0, int64_t count, int32_t *out)
{
    int rc = get_range(st_, v0, count, out);
    if (rc) return rc;
    for (int64_t i = 0; i < count; i++) out[i] = st_infinite(out[i]);
    return PSI_OK;
}

int Solver::get_strategy(int32_t *out)
{
    int rc = set_device();
    if (rc) return rc;
    PSI_CUDA_TRY(cudaMemcpyAsync(out, strat_, 4 * (size_t)n_, cudaMemcpyDeviceToHost, stream_));
    PSI_CUDA_TRY(cudaStreamSynchronize(stream_));
    return PSI_OK;
}

int Solver::get_solved(int32_t *out)
{
    int rc = set_device();
    if (rc) return rc;
    std::vector<uint8_t> s(n_);
    PSI_CUDA_TRY(cudaMemcpyAsync(s.data(), solved_, n_, cudaMemcpyDeviceToHost, stream_));
    PSI_CUDA_TRY(cudaStreamSynchronize(stream_));
    for (int32_t v = 0; v < n_; v++) out[v] = s[v];
    return PSI_OK;
}

int Solver::get_path_summary(int32_t *depth, int32_t *top, int32_t *count)
{
    if (!val_ready_) return fail(PSI_ERR_STATE, "get_path_summary before compute_valuation");
    int rc = set_device();
    if (rc) return rc;
    std::vector<int32_t> st(n_);
    std::vector<PathNode> nd(n_);
    PSI_CUDA_TRY(cudaMemcpyAsync(st.data(), st_, 4 * (size_t)n_, cudaMemcpyDeviceToHost, stream_));
    PSI_CUDA_TRY(cudaMemcpyAsync(nd.data(), node_, sizeof(PathNode) * (size_t)n_, cudaMemcpyDeviceToHost, stream_));
    PSI_CUDA_TRY(cudaStreamSynchronize(stream_));
    for (int32_t v = 0; v < n_; v++) {
        const bool fin = st[v] >= 1;
        if (depth) depth[v] = fin ? st[v] : 0;
        if (top) top[v] = fin ? nd[v].rmax : -1;
        if (count) count[v] = fin ? nd[v].rcnt : 0;
    }
    return PSI_OK;
}

int Solver::set_strategy(const int32_t *in)
{
    int rc = set_device();
    if (rc) return rc;
    // every entry must be one of the vertex's successors, or the sink for Even
    std::vector<int32_t> own(n_), off(n_ + 1), tgt(m_);
    std::vector<int8_t> own8(n_);
    PSI_CUDA_TRY(cudaMemcpyAsync(own8.data(), owner_, n_, cudaMemcpyDeviceToHost, stream_));
    PSI_CUDA_TRY(cudaMemcpyAsync(off.data(), off_, 4 * ((size_t)n_ + 1), cudaMemcpyDeviceToHost, stream_));
    if (m_) PSI_CUDA_TRY(cudaMemcpyAsync(tgt.data(), tgt_, 4 * (size_t)m_, cudaMemcpyDeviceToHost, stream_));
    PSI_CUDA_TRY(cudaStreamSynchronize(stream_));
    for (int32_t v = 0; v < n_; v++) {
        int32_t t = in[v];
        bool ok = (t == -1 && own8[v] == 0);
        for (int32_t e = off[v]; !ok && e < off[v + 1]; e++) ok = (tgt[e] == t);
        if (!ok) return fail(PSI_ERR_INVALID, "strategy entry of vertex " + std::to_string(v) + " is not a successor");
    }
    PSI_CUDA_TRY(cudaMemcpyAsync(strat_, in, 4 * (size_t)n_, cudaMemcpyHostToDevice, stream_));
    reset_tracking();
    PSI_CUDA_TRY(cudaStreamSynchronize(stream_));
    strat_ready_ = true;
    tour_valid_ = false;
    return PSI_OK;
}

int Solver::get_valuation(int32_t v0, int32_t count, int32_t *out)
{
    if (!val_ready_) return fail(PSI_ERR_STATE, "get_valuation before compute_valuation");
    if (v0 < 0 || count < 0 || (int64_t)v0 + count > n_) return fail(PSI_ERR_INVALID, "vertex range out of bounds");
    int64_t d = (int64_t)max_pri_ + 1;
    int64_t bytes = 4 * d * count;
    if (count == 0) return PSI_OK;
    int rc = set_device();
    if (rc) return rc;
    int32_t *rows = nullptr;
    cudaError_t e = device_alloc((void **)&rows, (size_t)bytes, stream_);
    if (e != cudaSuccess) return fail(PSI_ERR_NOMEM, "valuation export buffer");
    launch_materialize(stream_, v0, count, (int32_t)d, st_, node_, rows, &dw_->err);
    PSI_CUDA_TRY(cudaMemcpyAsync(out, rows, (size_t)bytes, cudaMemcpyDeviceToHost, stream_));
    PSI_CUDA_TRY(cudaFreeAsync(rows, stream_));
    return sync_and_check("get_valuation");
}

int Solver::solve(int32_t reset, int32_t *iters, int32_t *brs, int64_t max_evals)
{
    int32_t it = 0, br = 0;
    bool first = true;
    int rc = init_strat();
    if (rc) return rc;
    for (;;) {
        if (!first && reset) {
            rc = reset_opponent_strategy();
            if (rc) return rc;
        }
        for (;;) {
            rc = first ? compute_first_val() : compute_valuation();
            if (rc) return rc;
            br++;
            rc = mark_solved(1);
            if (rc) return rc;
            int64_t sw = 0;
            rc = switch_strategy(1, &sw);
            if (rc) return rc;
            if (sw == 0) break;
            if (max_evals > 0 && br >= max_evals) {
                *iters = it;
                *brs = br;
                return fail(PSI_ERR_LIMIT, "evaluation cap reached");
            }
        }
        first = false;
        rc = mark_solved(0);
        if (rc) return rc;
        it++;
        int64_t sw = 0;
        rc = switch_strategy(0, &sw);
        if (rc) return rc;
        if (sw == 0) break;
        if (max_evals > 0 && br >= max_evals) {
            *iters = it;
            *brs = br;
            return fail(PSI_ERR_LIMIT, "evaluation cap reached");
        }
    }
    *iters = it;
    *brs = br;
    return PSI_OK;
}

// solve_si (main.cpp:20-55) over the union with per-game accounting
// (launch_batch_account): the union's loops end when no game switches.
int Solver::solve_batch(int32_t *iters, int32_t *brs)
{
    if (!games_ || arena_) return fail(PSI_ERR_STATE, "not a batch");
    if (use_graph_) {   // the default: the whole loop as one graph launch
        std::vector<int4> st;
        int rc = solve_batch_graph(st);
        if (rc) return rc;
        for (int32_t k = 0; k < games_; k++) {
            brs[k] = st[k].x;
            iters[k] = st[k].y;
            if (!st[k].w) return fail(PSI_ERR_STATE, "batch loop ended with an unfinished game");
        }
        return PSI_OK;
    }
    int rc = init_strat();
    if (rc) return rc;
    PSI_CUDA_TRY(cudaMemsetAsync(gstate_, 0, 16 * (size_t)games_, stream_));
    PSI_CUDA_TRY(cudaMemsetAsync(gcount_, 0, 8 * (size_t)games_, stream_));
    for (;;) {
        for (;;) {
            rc = compute_valuation();
            if (rc) return rc;
            launch_batch_account(stream_, games_, 0, gstate_, gcount_);
            rc = mark_solved(1);
            if (rc) return rc;
            int64_t sw = 0;
            rc = switch_strategy(1, &sw);
            if (rc) return rc;
            launch_batch_account(stream_, games_, 1, gstate_, gcount_);
            if (sw == 0) break;
        }
        rc = mark_solved(0);
        if (rc) return rc;
        launch_batch_account(stream_, games_, 2, gstate_, gcount_);
        int64_t sw = 0;
        rc = switch_strategy(0, &sw);
        if (rc) return rc;
        launch_batch_account(stream_, games_, 3, gstate_, gcount_);
        if (sw == 0) break;
    }
    std::vector<int4> st((size_t)games_);
    PSI_CUDA_TRY(cudaMemcpyAsync(st.data(), gstate_, 16 * (size_t)games_, cudaMemcpyDeviceToHost, stream_));
    rc = sync_and_check("solve_batch");
    if (rc) return rc;
    for (int32_t k = 0; k < games_; k++) {
        brs[k] = st[k].x;
        iters[k] = st[k].y;
        if (!st[k].w) return fail(PSI_ERR_STATE, "batch loop ended with an unfinished game");
    }
    return PSI_OK;
}

// ---- serving arena ------------------------------------------------------

int Solver::init_arena(int32_t slots)
{
    set_extent(0);
    m_ = 0;
    max_pri_ = 0;
    np0_ = np_ = 0;
    const struct {
        void **ptr;
        size_t bytes;
    } arrays[] = {{(void **)&game_of_, 4 * (size_t)cap_n_},
                  {(void **)&gstate_, sizeof(int4) * (size_t)slots},
                  {(void **)&gcount_, sizeof(unsigned long long) * (size_t)slots},
                  {(void **)&gmask_, 4 * (size_t)slots}};
    for (const auto &a : arrays) {
        cudaError_t e = device_alloc(a.ptr, a.bytes, stream_);
        if (e != cudaSuccess) return fail(PSI_ERR_NOMEM, std::string("device allocation: ") + cudaGetErrorString(e));
        allocs_.push_back(*a.ptr);
    }
    games_ = slots;
    arena_ = true;
    PSI_CUDA_TRY(cudaMemsetAsync(solved_, 1, (size_t)cap_n_, stream_));          // every slot inert
    PSI_CUDA_TRY(cudaMemsetAsync(game_of_, 0xff, 4 * (size_t)cap_n_, stream_));   // -1: in no game
    PSI_CUDA_TRY(cudaMemsetAsync(st_, 0, 4 * (size_t)cap_n_, stream_));            // no finite depths
    launch_isolate_pairs(stream_, cap_n_ + 1, succ_);                              // no slot in the tour
    launch_move_extent(stream_, 0, 0, succ_);
    PSI_CUDA_TRY(cudaMemsetAsync(gstate_, 0, sizeof(int4) * (size_t)slots, stream_));
    PSI_CUDA_TRY(cudaMemsetAsync(gcount_, 0, sizeof(unsigned long long) * (size_t)slots, stream_));
    PSI_CUDA_TRY(cudaMemsetAsync(gmask_, 0, 4 * (size_t)slots, stream_));
    PSI_CUDA_TRY(cudaStreamSynchronize(stream_));
    strat_ready_ = true;
    return PSI_OK;
}

// Places the games admitted in one step: each game's arrays are copied as
// they are into a device staging union (no host packing), shifted to union
// numbering on the device, given one reverse-CSR build and placed by one
// launch.  The tour stays valid: placed vertices start as isolated pairs and
// dirty parents, which the next evaluation relinks.
int Solver::arena_add(const std::vector<const HostGame *> &gs, const std::vector<int32_t> &vb,
                      const std::vector<int32_t> &eb, const std::vector<int32_t> &slot, int32_t extent)
{
    if (!arena_) return fail(PSI_ERR_STATE, "not an arena");
    const int32_t K = (int32_t)gs.size();
    if (K == 0) return PSI_OK;
    if ((int32_t)vb.size() != K || (int32_t)eb.size() != K || (int32_t)slot.size() != K || extent > cap_n_)
        return fail(PSI_ERR_INVALID, "arena placement lists disagree");
    int64_t n = 0, m = 0;
    int32_t top = 0;
    // per-game table: ub[K+1], ue[K+1], vb[K], eb[K], slot[K]
    std::vector<int32_t> table(5 * (size_t)K + 2);
    int32_t *ub = table.data(), *ue = ub + K + 1;
    for (int32_t k = 0; k < K; k++) {
        const HostGame &g = *gs[k];
        if (g.n <= 0 || slot[k] < 0 || slot[k] >= games_ || vb[k] < 0 || eb[k] < 0 ||
            (int64_t)vb[k] + g.n + 1 > extent || (int64_t)eb[k] + g.m > cap_m_)
            return fail(PSI_ERR_INVALID, "arena placement out of range");
        ub[k] = (int32_t)n;
        ue[k] = (int32_t)m;
        n += g.n;
        m += g.m;
        top = g.max_pri > top ? g.max_pri : top;
        table[2 * (size_t)K + 2 + k] = vb[k];
        table[3 * (size_t)K + 2 + k] = eb[k];
        table[4 * (size_t)K + 2 + k] = slot[k];
    }
    if (2 * n + 2 > INT32_MAX || m > INT32_MAX) return fail(PSI_ERR_TOO_LARGE, "admission too large for int32 ids");
    ub[K] = (int32_t)n;
    ue[K] = (int32_t)m;
    int rc = set_device();
    if (rc) return rc;
    int32_t *d_tab = nullptr, *u_owner = nullptr, *u_pri = nullptr, *u_off = nullptr, *u_tgt = nullptr,
            *u_roff = nullptr, *u_rsrc = nullptr;
    int32_t **bufs[] = {&d_tab, &u_owner, &u_pri, &u_off, &u_tgt, &u_roff, &u_rsrc};
    const size_t sizes[] = {4 * table.size(),   4 * (size_t)n,       4 * (size_t)n,      4 * ((size_t)n + 1),
                            4 * (size_t)m,      4 * ((size_t)n + 1), 4 * (size_t)m};
    cudaError_t e = cudaSuccess;
    int64_t mr = 0;
    int ce = 0;
    for (int i = 0; i < 7 && e == cudaSuccess; i++) e = device_alloc((void **)bufs[i], sizes[i], stream_);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(d_tab, table.data(), sizes[0], cudaMemcpyHostToDevice, stream_);
    for (int32_t k = 0; k < K && e == cudaSuccess; k++) {
        const HostGame &g = *gs[k];
        const size_t nb = 4 * (size_t)g.n;
        e = cudaMemcpyAsync(u_owner + ub[k], g.owner.data(), nb, cudaMemcpyHostToDevice, stream_);
        if (e == cudaSuccess) e = cudaMemcpyAsync(u_pri + ub[k], g.priority.data(), nb, cudaMemcpyHostToDevice, stream_);
        if (e == cudaSuccess) e = cudaMemcpyAsync(u_off + ub[k], g.offsets.data(), nb, cudaMemcpyHostToDevice, stream_);
        if (e == cudaSuccess && g.m)
            e = cudaMemcpyAsync(u_tgt + ue[k], g.targets.data(), 4 * (size_t)g.m, cudaMemcpyHostToDevice, stream_);
    }
    if (e == cudaSuccess) {
        launch_union_fixup(stream_, (int32_t)n, m, K, d_tab, d_tab + K + 1, u_off, u_tgt);
        ce = build_reverse_csr(stream_, (int32_t)n, m, u_off, u_tgt, u_roff, u_rsrc, &mr);
    }
    if (e == cudaSuccess && !ce) {
        // with full evaluations only, the unreached list is rebuilt before its next use; after a
        // patch mark_solved reads it (the new vertices are appended by the patch)
        if (incremental_ == PSI_INCR_OFF) e = cudaMemsetAsync(&dw_->ucount, 0, sizeof(int32_t), stream_);
        if (extent != n_) launch_move_extent(stream_, n_, extent, succ_);
        const int32_t *vbd = d_tab + 2 * K + 2, *ebd = d_tab + 3 * K + 2, *sld = d_tab + 4 * K + 2;
        launch_arena_place(stream_, (int32_t)n, K, d_tab, vbd, ebd, sld, u_owner, u_pri, u_off, u_tgt, u_roff, u_rsrc,
                           owner_, pri_, off_, tgt_, rev_off_, rev_src_, strat_, st_, solved_, game_of_, gstate_,
                           gcount_, succ_, dirty_, need_, changes());
        if (e == cudaSuccess) e = cudaGetLastError();
    }
    for (int i = 0; i < 7; i++)
        if (*bufs[i]) cudaFreeAsync(*bufs[i], stream_);
    if (ce) return fail(PSI_ERR_CUDA, std::string("reverse CSR: ") + cudaGetErrorString((cudaError_t)ce));
    if (e != cudaSuccess) return fail(PSI_ERR_CUDA, std::string("arena_add: ") + cudaGetErrorString(e));
    if (top > max_pri_) max_pri_ = top;
    set_extent(extent);
    return sync_and_check("arena_add");
}

// Retires games: their ranges become inert and leave the tour (one
// synchronisation for all of them).
int Solver::arena_remove(const std::vector<int32_t> &vb, const std::vector<int32_t> &count,
                         const std::vector<int32_t> &slot, int32_t extent)
{
    if (!arena_) return fail(PSI_ERR_STATE, "not an arena");
    const size_t K = vb.size();
    if (count.size() != K || slot.size() != K || extent > cap_n_) return fail(PSI_ERR_INVALID, "arena lists disagree");
    for (size_t k = 0; k < K; k++)
        if (slot[k] < 0 || slot[k] >= games_ || vb[k] < 0 || count[k] < 0 || (int64_t)vb[k] + count[k] > cap_n_)
            return fail(PSI_ERR_INVALID, "arena range out of range");
    int rc = set_device();
    if (rc) return rc;
    for (size_t k = 0; k < K; k++) {
        launch_arena_clear(stream_, vb[k], count[k], solved_, game_of_, st_, succ_, dirty_);
        PSI_CUDA_TRY(cudaMemsetAsync(gstate_ + slot[k], 0, sizeof(int4), stream_));
    }
    // the retired vertices left in the unreached list are solved: mark_solved passes them by
    if (incremental_ == PSI_INCR_OFF) PSI_CUDA_TRY(cudaMemsetAsync(&dw_->ucount, 0, sizeof(int32_t), stream_));
    if (extent != n_) launch_move_extent(stream_, n_, extent, succ_);
    set_extent(extent);
    return sync_and_check("arena_remove");
}

int Solver::arena_export(int32_t vb, int32_t count, int32_t *strategy, int32_t *infinite)
{
    if (vb < 0 || count < 0 || (int64_t)vb + count > n_) return fail(PSI_ERR_INVALID, "arena range out of range");
    if (count == 0) return PSI_OK;
    int32_t *out = nullptr;
    cudaError_t e = device_alloc((void **)&out, 8 * (size_t)count, stream_);
    if (e != cudaSuccess) return fail(PSI_ERR_NOMEM, "arena export buffer");
    launch_arena_export(stream_, vb, count, strat_, st_, out);
    e = cudaMemcpyAsync(strategy, out, 4 * (size_t)count, cudaMemcpyDeviceToHost, stream_);
    if (e == cudaSuccess) e = cudaMemcpyAsync(infinite, out + count, 4 * (size_t)count, cudaMemcpyDeviceToHost, stream_);
    cudaFreeAsync(out, stream_);
    if (e != cudaSuccess) return fail(PSI_ERR_CUDA, std::string("arena export: ") + cudaGetErrorString(e));
    return sync_and_check("arena_export");
}

// Player lists of the vertices that belong to games (Even's first).
int Solver::arena_rebuild_lists()
{
    int rc = set_device();
    if (rc) return rc;
    PSI_CUDA_TRY(cudaMemsetAsync(&dw_->sinkcount, 0, sizeof(int32_t), stream_));
    launch_build_plist(stream_, n_, 0, owner_, game_of_, plist_, &dw_->sinkcount);
    rc = sync_and_check("arena_rebuild_lists");
    if (rc) return rc;
    np0_ = hw_->sinkcount;
    launch_build_plist(stream_, n_, 1, owner_, game_of_, plist_, &dw_->sinkcount);   // appends after Even's
    rc = sync_and_check("arena_rebuild_lists");
    if (rc) return rc;
    np_ = hw_->sinkcount;
    return PSI_OK;
}

// One solve_si step (main.cpp:20-55) of every resident game, each by its own
// state machine (launch_serve_account): evaluate all, switch Odd in all, then
// mark_solved(Even) and switch Even only in the games whose Odd made no
// strict improvement in this step.
int Solver::arena_step(bool reset, std::vector<int32_t> &done, std::vector<int32_t> &iters,
                       std::vector<int32_t> &brs)
{
    done.clear();
    iters.clear();
    brs.clear();
    if (!arena_) return fail(PSI_ERR_STATE, "not an arena");
    if (n_ == 0 || np_ == 0) return PSI_OK;
    int rc = compute_valuation();
    if (rc) return rc;
    launch_serve_account(stream_, games_, 0, gstate_, gcount_, gmask_);
    int32_t *mask = gmask_;
    gmask_ = nullptr;                       // Odd's step: every resident game
    rc = mark_solved(1);
    int64_t sw = 0;
    if (!rc) rc = switch_strategy(1, &sw);
    gmask_ = mask;
    if (rc) return rc;
    launch_serve_account(stream_, games_, 1, gstate_, gcount_, gmask_);
    rc = mark_solved(0);                    // Even's step: games with gmask set
    if (!rc) rc = switch_strategy(0, &sw);
    if (rc) return rc;
    if (reset)
        launch_serve_reset_odd(stream_, np_ - np0_, plist_ + np0_, game_of_, gmask_, gcount_, off_, tgt_, strat_,
                               dirty_, need_, changes());
    launch_serve_account(stream_, games_, 2, gstate_, gcount_, gmask_);
    std::vector<int4> st((size_t)games_);
    PSI_CUDA_TRY(cudaMemcpyAsync(st.data(), gstate_, sizeof(int4) * (size_t)games_, cudaMemcpyDeviceToHost, stream_));
    rc = sync_and_check("arena_step");
    if (rc) return rc;
    for (int32_t k = 0; k < games_; k++)
        if ((st[k].z & 1) && (st[k].z & 2)) {
            done.push_back(k);
            iters.push_back(st[k].y);
            brs.push_back(st[k].x);
        }
    return PSI_OK;
}

}  // namespace psi
