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

int Solver::create(const HostGame &g, const psi_options &opt, Solver **out)
{
    *out = nullptr;
    if (g.n <= 0) return fail(PSI_ERR_INVALID, "game has no vertices");
    if (2 * (int64_t)g.n + 2 > INT32_MAX) return fail(PSI_ERR_TOO_LARGE, "n too large for int32 tour ids");
    if (opt.valuation_mode != PSI_VAL_PATH) return fail(PSI_ERR_INVALID, "unknown valuation_mode");
    if (opt.sublist_len < 2) return fail(PSI_ERR_INVALID, "sublist_len must be >= 2");
    int ndev = 0;
    cudaError_t e = cudaGetDeviceCount(&ndev);
    if (e != cudaSuccess || ndev == 0) return fail(PSI_ERR_NO_DEVICE, "no CUDA device available");
    if (opt.device < 0 || opt.device >= ndev) return fail(PSI_ERR_INVALID, "device ordinal out of range");
    Solver *s = new Solver();
    s->device_ = opt.device;
    s->timing_ = opt.timing != 0;
    s->stride_ = opt.sublist_len;
    int rc = s->alloc(g, opt);
    if (rc) {
        delete s;
        return rc;
    }
    *out = s;
    return PSI_OK;
}

int Solver::alloc(const HostGame &g, const psi_options &)
{
    int rc = set_device();
    if (rc) return rc;
    n_ = g.n;
    m_ = g.m;
    max_pri_ = g.max_pri;
    L_ = 2 * (int64_t)n_ + 2;
    // heads at node j*stride for j < nsub-1, plus the list start (node L-1)
    nsub_ = (int32_t)(ceil_div(L_ - 1, stride_) + 1);
    game_ = &g;
    PSI_CUDA_TRY(cudaStreamCreateWithFlags(&stream_, cudaStreamNonBlocking));
    PSI_CUDA_TRY(cudaEventCreate(&ev0_));
    PSI_CUDA_TRY(cudaEventCreate(&ev1_));

    auto dalloc = [&](void **p, size_t bytes) -> int {
        cudaError_t e = cudaMalloc(p, bytes ? bytes : 16);
        if (e != cudaSuccess) return fail(PSI_ERR_NOMEM, std::string("cudaMalloc: ") + cudaGetErrorString(e));
        allocs_.push_back(*p);
        return PSI_OK;
    };
#define PSI_DALLOC(ptr, bytes)                                  \
    do {                                                        \
        int r__ = dalloc((void **)&(ptr), (size_t)(bytes));     \
        if (r__) return r__;                                    \
    } while (0)
    PSI_DALLOC(owner_, n_);
    PSI_DALLOC(pri_, 4 * (size_t)n_);
    PSI_DALLOC(off_, 4 * ((size_t)n_ + 1));
    PSI_DALLOC(tgt_, 4 * (size_t)m_);
    PSI_DALLOC(strat_, 4 * (size_t)n_);
    PSI_DALLOC(st_, 4 * (size_t)n_);
    PSI_DALLOC(solved_, n_);
    PSI_DALLOC(pp_, 8 * (size_t)n_);
    PSI_DALLOC(succ_, 4 * (size_t)L_);
    PSI_DALLOC(hsucc_, 4 * (size_t)nsub_);
    PSI_DALLOC(ulist_, 4 * (size_t)n_);
    PSI_DALLOC(vloc_, 8 * (size_t)n_);
    PSI_DALLOC(redA_, 8 * (size_t)nsub_);
    PSI_DALLOC(redB_, 8 * (size_t)nsub_);
    PSI_DALLOC(jA_, 8 * (size_t)n_);
    PSI_DALLOC(jB_, 8 * (size_t)n_);
    PSI_DALLOC(dw_, sizeof(Words));
#undef PSI_DALLOC
    PSI_CUDA_TRY(cudaMallocHost((void **)&hw_, sizeof(Words)));

    std::vector<int8_t> own8(g.owner.begin(), g.owner.end());
    PSI_CUDA_TRY(cudaMemcpyAsync(owner_, own8.data(), n_, cudaMemcpyHostToDevice, stream_));
    PSI_CUDA_TRY(cudaMemcpyAsync(pri_, g.priority.data(), 4 * (size_t)n_, cudaMemcpyHostToDevice, stream_));
    PSI_CUDA_TRY(cudaMemcpyAsync(off_, g.offsets.data(), 4 * ((size_t)n_ + 1), cudaMemcpyHostToDevice, stream_));
    if (m_) PSI_CUDA_TRY(cudaMemcpyAsync(tgt_, g.targets.data(), 4 * (size_t)m_, cudaMemcpyHostToDevice, stream_));
    PSI_CUDA_TRY(cudaMemsetAsync(solved_, 0, n_, stream_));
    PSI_CUDA_TRY(cudaMemsetAsync(st_, 0, 4 * (size_t)n_, stream_));
    PSI_CUDA_TRY(cudaMemsetAsync(dw_, 0, sizeof(Words), stream_));
    PSI_CUDA_TRY(cudaStreamSynchronize(stream_));
    game_ = nullptr;
    return PSI_OK;
}

Solver::~Solver()
{
    cudaSetDevice(device_);
    if (stream_) cudaStreamSynchronize(stream_);
    for (void *p : allocs_) cudaFree(p);
    if (hw_) cudaFreeHost(hw_);
    if (ev0_) cudaEventDestroy(ev0_);
    if (ev1_) cudaEventDestroy(ev1_);
    if (stream_) cudaStreamDestroy(stream_);
}

int Solver::sync_and_check(const char *what)
{
    PSI_CUDA_TRY(cudaGetLastError());
    PSI_CUDA_TRY(cudaMemcpyAsync(hw_, dw_, sizeof(Words), cudaMemcpyDeviceToHost, stream_));
    cudaError_t e = cudaStreamSynchronize(stream_);
    if (e != cudaSuccess) return fail(PSI_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
    if (hw_->err) {
        uint32_t bits = hw_->err;
        cudaMemsetAsync(dw_, 0, sizeof(Words), stream_);
        cudaStreamSynchronize(stream_);
        return fail(PSI_ERR_LIMIT, std::string(what) + ": device step cap reached (bits " + std::to_string(bits) + ")");
    }
    return PSI_OK;
}

int Solver::init_strat()
{
    int rc = set_device();
    if (rc) return rc;
    launch_init_strat(stream_, n_, owner_, off_, tgt_, strat_, st_);
    PSI_CUDA_TRY(cudaMemsetAsync(solved_, 0, n_, stream_));
    rc = sync_and_check("init_strat");
    if (rc) return rc;
    strat_ready_ = true;
    val_ready_ = false;
    return PSI_OK;
}

int Solver::reset_opponent_strategy()
{
    if (!strat_ready_) return fail(PSI_ERR_STATE, "reset_opponent_strategy before init_strat");
    int rc = set_device();
    if (rc) return rc;
    launch_reset_odd(stream_, n_, owner_, off_, tgt_, strat_);
    return sync_and_check("reset_opponent_strategy");
}

int Solver::compute_valuation()
{
    if (!strat_ready_) return fail(PSI_ERR_STATE, "compute_valuation before init_strat");
    int rc = set_device();
    if (rc) return rc;
    if (timing_) PSI_CUDA_TRY(cudaEventRecord(ev0_, stream_));
    // 1. Euler tour of the sink tree
    launch_tour_init(stream_, n_, succ_, vloc_);
    launch_tour_link(stream_, n_, strat_, solved_, succ_);
    // 2. Helman-JaJa sublists + Wyllie over the reduced list
    launch_pick_heads(stream_, L_, nsub_, stride_, succ_, hsucc_);
    launch_walk_sublists(stream_, nsub_, n_, L_, succ_, hsucc_, vloc_, redA_, &dw_->err);
    int rounds = ceil_log2(nsub_) + 1;
    int2 *in = redA_, *out = redB_;
    for (int r = 0; r < rounds; r++) {
        launch_wyllie_round(stream_, nsub_, in, out);
        std::swap(in, out);
    }
    // 3. broadcast depths; collect the vertices the sink does not reach
    PSI_CUDA_TRY(cudaMemsetAsync(&dw_->ucount, 0, sizeof(int32_t), stream_));
    launch_broadcast_depth(stream_, n_, vloc_, in, strat_, pri_, solved_, st_, pp_, ulist_, &dw_->ucount);
    rc = sync_and_check("compute_valuation (ranking)");
    if (rc) return rc;
    int32_t nu = hw_->ucount;
    last_unreached_ = nu;
    // 4. cycle parity by pointer jumping over the unreached vertices
    if (nu > 0) {
        launch_jump_init(stream_, nu, ulist_, strat_, pri_, jA_, &dw_->err);
        int jr = ceil_log2(nu) + 1;
        int2 *ja = jA_, *jb = jB_;
        for (int r = 0; r < jr; r++) {
            launch_jump_round(stream_, nu, ulist_, solved_, ja, jb);
            std::swap(ja, jb);
        }
        launch_jump_finish(stream_, nu, ulist_, solved_, ja, st_);
    }
    if (timing_) PSI_CUDA_TRY(cudaEventRecord(ev1_, stream_));
    rc = sync_and_check("compute_valuation");
    if (rc) return rc;
    if (timing_) {
        float ms = 0;
        PSI_CUDA_TRY(cudaEventElapsedTime(&ms, ev0_, ev1_));
        times_.eval_ms += ms;
    }
    times_.evals++;
    val_ready_ = true;
    return PSI_OK;
}

int Solver::mark_solved(int32_t player)
{
    if (player != 0 && player != 1) return fail(PSI_ERR_INVALID, "player must be 0 or 1");
    if (!val_ready_) return fail(PSI_ERR_STATE, "mark_solved before compute_valuation");
    int rc = set_device();
    if (rc) return rc;
    launch_mark_solved(stream_, n_, player, st_, solved_);
    PSI_CUDA_TRY(cudaGetLastError());
    return PSI_OK;   // ordered on the stream before the next call
}

int Solver::switch_strategy(int32_t player, int64_t *switched)
{
    if (player != 0 && player != 1) return fail(PSI_ERR_INVALID, "player must be 0 or 1");
    if (!val_ready_) return fail(PSI_ERR_STATE, "switch_strategy before compute_valuation");
    int rc = set_device();
    if (rc) return rc;
    PSI_CUDA_TRY(cudaMemsetAsync(&dw_->count, 0, sizeof(unsigned long long), stream_));
    if (timing_) PSI_CUDA_TRY(cudaEventRecord(ev0_, stream_));
    launch_switch(stream_, n_, player, owner_, off_, tgt_, strat_, st_, pp_, &dw_->count, &dw_->err);
    if (timing_) PSI_CUDA_TRY(cudaEventRecord(ev1_, stream_));
    rc = sync_and_check("switch_strategy");
    if (rc) return rc;
    if (timing_) {
        float ms = 0;
        PSI_CUDA_TRY(cudaEventElapsedTime(&ms, ev0_, ev1_));
        times_.switch_ms += ms;
    }
    times_.switches++;
    if (switched) *switched = (int64_t)hw_->count;
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
    if (player != 0 && player != 1) return fail(PSI_ERR_INVALID, "player must be 0 or 1");
    std::vector<int32_t> inf(n_);
    int rc = get_infinite(inf.data());
    if (rc) return rc;
    out.clear();
    for (int32_t v = 0; v < n_; v++) {
        bool w0 = inf[v] == 1;
        if ((player == 0 && w0) || (player == 1 && !w0)) out.push_back(v);
    }
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
    PSI_CUDA_TRY(cudaStreamSynchronize(stream_));
    strat_ready_ = true;
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
    cudaError_t e = cudaMallocAsync((void **)&rows, (size_t)bytes, stream_);
    if (e != cudaSuccess) return fail(PSI_ERR_NOMEM, "valuation export buffer");
    launch_materialize(stream_, v0, count, (int32_t)d, st_, pp_, rows, &dw_->err);
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

}  // namespace psi
