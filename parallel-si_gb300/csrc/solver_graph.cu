// solver_graph.cu -- solve_si (main.cpp:20-55) as one CUDA graph.
//
// The host-driven loop (Solver::solve) synchronises after every evaluation
// and every switch step to read the switch count that decides what comes
// next.  Here the decision moves to the device: one SI step -- an optional
// reset of Odd's strategy, an evaluation, mark_solved(Odd) and Odd's switch,
// then mark_solved(Even) and Even's switch -- is captured once as the body of
// a conditional "while" node, and small control kernels read the switch
// counts and set gate words (which kernels of the next pass do work) and,
// when the loop is over, the node's condition.  A whole solve is one graph
// launch and one synchronisation.  The kernels are the same as the host
// loop's; gated ones return at once when their gate word is 0.
#include <string>
#include <vector>

#include "device_common.cuh"
#include "kernels.h"
#include "psi_internal.h"
#include "solver.h"

namespace psi {

namespace {

// after an evaluation: the tour is valid for updates (and the next
// evaluation may be a patch), one more evaluation
__global__ void k_ctl_evaluated(GraphCtl *c, uint32_t *err)
{
    c->full = 0;
    c->incr = 1;
    c->try_patch = c->patch_on;
    c->reset = 0;
    c->quiet = 0;
    c->brs++;
    if (c->inject_at > 0 && c->brs == c->inject_at) atomicOr(err, c->inject_bits);
}

// after Odd's switch: Even moves in this step iff Odd made no strict improvement
__global__ void k_ctl_odd(GraphCtl *c, const unsigned long long *sw) { c->even = (sw[3] == 0) ? 1 : 0; }

// after Even's (gated) switch: iteration count, termination, reset, caps.
// A set bit of the device error word ends the loop after this pass: the
// state it left may be inconsistent, and later passes must not build on it.
__global__ void k_ctl_even(GraphCtl *c, const unsigned long long *sw, const uint32_t *err,
                           cudaGraphConditionalHandle loop, int32_t reset_variant, int32_t guard)
{
    if (*(volatile const uint32_t *)err) {
        c->stop = GraphCtl::kDeviceError;
        cudaGraphSetConditional(loop, 0);
        return;
    }
    bool go = true;
    if (c->even) {
        c->iters++;
        if (sw[3] == 0) {
            c->stop = GraphCtl::kConverged;
            go = false;
        } else if (reset_variant) {   // main.cpp:25-26: Odd starts the next iteration afresh
            c->reset = 1;
            c->full = 1;              // many Odd strategies change: rebuild the tour
            c->incr = 0;
            c->try_patch = 0;         // and no switch step lists those changes
        }
    }
    if (go && c->max_evals > 0 && c->brs >= c->max_evals) {
        c->stop = GraphCtl::kEvalCap;
        go = false;
    }
    if (go && c->brs >= guard) {
        c->stop = GraphCtl::kRunaway;
        go = false;
    }
    if (!go) cudaGraphSetConditional(loop, 0);
}

// A solve that needs more evaluations than this is treated as a runaway (the
// loop runs on the device and must end by itself): 64 per vertex plus a
// margin, between 2^14 and 2^20.  Random games of 2^24 vertices need under
// 100; a caller expecting more passes max_evals or uses the host loop.
inline int32_t eval_guard(int64_t n)
{
    const int64_t g = 64 * (n + 64);
    return (int32_t)(g < (1 << 14) ? (1 << 14) : (g > (1 << 20) ? (1 << 20) : g));
}

}  // namespace

// Opens the full evaluation's conditional node iff this evaluation is not a
// patch (its gate word was set by k_patch_begin / k_patch_collect).
__global__ void k_eval_cond(const GraphCtl *c, cudaGraphConditionalHandle h) { cudaGraphSetConditional(h, c->eval ? 1 : 0); }

// One SI step captured into the loop body `body`, in three pieces: (A) Odd's
// reset and the patch kernels, then a kernel that sets the condition of (B),
// a conditional "if" node holding the full evaluation, so that a patched
// evaluation launches none of its kernels; (C) the rest of the step.
int Solver::enqueue_step(cudaGraph_t body, cudaGraphConditionalHandle loop, bool reset)
{
    const cudaStreamCaptureMode mode = cudaStreamCaptureModeThreadLocal;
    cudaGraphConditionalHandle evalc;
    PSI_CUDA_TRY(cudaGraphConditionalHandleCreate(&evalc, body, 1, 0));
    auto abort_capture = [&](int rc) {
        cudaGraph_t g = nullptr;
        cudaStreamEndCapture(stream_, &g);
        return rc;
    };

    // (A)
    PSI_CUDA_TRY(cudaStreamBeginCaptureToGraph(stream_, body, nullptr, nullptr, 0, mode));
    launch_reset_odd(stream_, n_, owner_, off_, tgt_, strat_, &ctl_->reset, need_);
    int rc = enqueue_patch(false);
    if (rc) return abort_capture(rc);
    count_launch();
    k_eval_cond<<<1, 1, 0, stream_>>>(ctl_, evalc);
    cudaStreamCaptureStatus status;
    const cudaGraphNode_t *deps = nullptr;
    size_t ndeps = 0;
    cudaError_t e = cudaStreamGetCaptureInfo(stream_, &status, nullptr, nullptr, &deps, nullptr, &ndeps);
    if (e != cudaSuccess) return abort_capture(fail(PSI_ERR_CUDA, std::string("capture info: ") + cudaGetErrorString(e)));
    std::vector<cudaGraphNode_t> tail(deps, deps + ndeps);
    cudaGraph_t g = nullptr;
    PSI_CUDA_TRY(cudaStreamEndCapture(stream_, &g));

    // (B) the full evaluation (as compute_valuation), inside the "if" node
    cudaGraphNodeParams ip = {};
    ip.type = cudaGraphNodeTypeConditional;
    ip.conditional.handle = evalc;
    ip.conditional.type = cudaGraphCondTypeIf;
    ip.conditional.size = 1;
    cudaGraphNode_t ifnode;
    PSI_CUDA_TRY(cudaGraphAddNode(&ifnode, body, tail.data(), nullptr, tail.size(), &ip));
    PSI_CUDA_TRY(cudaStreamBeginCaptureToGraph(stream_, ip.conditional.phGraph_out[0], nullptr, nullptr, 0, mode));
    const long long full_before = launch_count();
    rc = enqueue_full(false);
    graph_full_launches_ = launch_count() - full_before;
    if (rc) return abort_capture(rc);
    PSI_CUDA_TRY(cudaStreamEndCapture(stream_, &g));

    // (C); a batch also advances every game's own solve_si counts
    // (k_batch_account, at the points where the host loop calls it), and its
    // switch steps add each game's strict improvements to gcount_
    const bool batch = games_ > 0 && !arena_;
    PSI_CUDA_TRY(cudaStreamBeginCaptureToGraph(stream_, body, &ifnode, nullptr, 1, mode));
    count_launch();
    k_ctl_evaluated<<<1, 1, 0, stream_>>>(ctl_, &dw_->err);
    if (batch) launch_batch_account(stream_, games_, 0, gstate_, gcount_);
    // Odd: mark_solved(1), switch(1)
    launch_mark_solved(stream_, &dw_->ucount, ulist_, 1, st_, solved_, dirty_, nullptr, nullptr, nullptr,
                       &ctl_->mfrom[1], &ctl_->mdone);
    e = cudaMemsetAsync(dw_->sw, 0, sizeof(dw_->sw), stream_);
    if (e != cudaSuccess) return abort_capture(fail(PSI_ERR_CUDA, std::string("memset: ") + cudaGetErrorString(e)));
    int32_t *todo = reinterpret_cast<int32_t *>(jB_);   // free until the next cycle pass
    unsigned long long *gc = batch ? gcount_ : nullptr;
    launch_switch(stream_, np_ - np0_, plist_ + np0_, 1, off_, tgt_, strat_, st_, key_, node_, dw_->sw,
                  batch ? game_of_ : nullptr, gc, nullptr, dirty_, &dw_->err, nullptr, need_, todo, &dw_->cnt[2],
                  changes(), tie_, watch_, skip_, switch_warp_, &dw_->claim, arena_ ? nullptr : owner_, n_);
    if (batch) launch_batch_account(stream_, games_, 1, gstate_, gcount_);
    count_launch();
    k_ctl_odd<<<1, 1, 0, stream_>>>(ctl_, dw_->sw);
    // Even, when Odd made no strict improvement: mark_solved(0), switch(0)
    launch_mark_solved(stream_, &dw_->ucount, ulist_, 0, st_, solved_, dirty_, nullptr, nullptr, &ctl_->even,
                       &ctl_->mfrom[0], &ctl_->mdone);
    if (batch) launch_batch_account(stream_, games_, 2, gstate_, gcount_, &ctl_->even);
    e = cudaMemsetAsync(dw_->sw, 0, sizeof(dw_->sw), stream_);
    if (e != cudaSuccess) return abort_capture(fail(PSI_ERR_CUDA, std::string("memset: ") + cudaGetErrorString(e)));
    launch_switch(stream_, np0_, plist_, 0, off_, tgt_, strat_, st_, key_, node_, dw_->sw,
                  batch ? game_of_ : nullptr, gc, nullptr, dirty_, &dw_->err, &ctl_->even, need_, todo,
                  &dw_->cnt[2], changes(), tie_, watch_, skip_, switch_warp_, &dw_->claim,
                  arena_ ? nullptr : owner_, n_);
    if (batch) launch_batch_account(stream_, games_, 3, gstate_, gcount_, &ctl_->even);
    count_launch();
    k_ctl_even<<<1, 1, 0, stream_>>>(ctl_, dw_->sw, &dw_->err, loop, reset ? 1 : 0, eval_guard(n_));
    e = cudaGetLastError();
    if (e != cudaSuccess) return abort_capture(fail(PSI_ERR_CUDA, std::string("step launch: ") + cudaGetErrorString(e)));
    PSI_CUDA_TRY(cudaStreamEndCapture(stream_, &g));
    return PSI_OK;
}

int Solver::build_graph(bool reset)
{
    if (graph_exec_) {
        cudaGraphExecDestroy(graph_exec_);
        graph_exec_ = nullptr;
    }
    if (graph_) {
        cudaGraphDestroy(graph_);
        graph_ = nullptr;
    }
    PSI_CUDA_TRY(cudaGraphCreate(&graph_, 0));
    cudaGraphConditionalHandle loop;
    PSI_CUDA_TRY(cudaGraphConditionalHandleCreate(&loop, graph_, 1, cudaGraphCondAssignDefault));
    cudaGraphNodeParams cp = {};
    cp.type = cudaGraphNodeTypeConditional;
    cp.conditional.handle = loop;
    cp.conditional.type = cudaGraphCondTypeWhile;
    cp.conditional.size = 1;
    cudaGraphNode_t node;
    PSI_CUDA_TRY(cudaGraphAddNode(&node, graph_, nullptr, nullptr, 0, &cp));
    cudaGraph_t body = cp.conditional.phGraph_out[0];
    const long long before = launch_count();
    int rc = enqueue_step(body, loop, reset);
    graph_step_launches_ = launch_count() - before;
    if (rc) return rc;
    PSI_CUDA_TRY(cudaGraphInstantiate(&graph_exec_, graph_, 0));
    graph_reset_ = reset;
    return PSI_OK;
}

// One graph launch of the solve loop from init_strat; *out receives the
// loop's control words at the end.  With gstate_out (a batch), the per-game
// states are read back in the same synchronisation.
int Solver::run_graph(bool reset, int64_t max_evals, GraphCtl *out, int4 *gstate_out)
{
    int rc = init_strat();
    if (rc) return rc;
    const unsigned long long patches_before = hw_->patch[0];   // as of init_strat's synchronisation
    if (!graph_exec_ || graph_reset_ != reset) {
        rc = build_graph(reset);
        if (rc) return rc;
    }
    GraphCtl init;
    init.full = 1;   // init_strat: the first evaluation builds the tour
    init.quiet = 1;  // and every need flag is set
    init.patch_on = incremental_ != PSI_INCR_OFF ? 1 : 0;
    init.max_evals = max_evals > 0 && max_evals < INT32_MAX ? (int32_t)max_evals : 0;
    init.inject_at = inject_at_;
    init.inject_bits = inject_bits_;
    PSI_CUDA_TRY(cudaMemcpyAsync(ctl_, &init, sizeof init, cudaMemcpyHostToDevice, stream_));
    PSI_CUDA_TRY(cudaGraphLaunch(graph_exec_, stream_));
    PSI_CUDA_TRY(cudaMemcpyAsync(out, ctl_, sizeof *out, cudaMemcpyDeviceToHost, stream_));
    if (gstate_out)
        PSI_CUDA_TRY(cudaMemcpyAsync(gstate_out, gstate_, sizeof(int4) * (size_t)games_, cudaMemcpyDeviceToHost,
                                     stream_));
    // the counts of the passes that ran are kept even when a pass failed
    rc = sync_and_check("solve (graph)");
    if (rc && rc != PSI_ERR_LIMIT) return rc;
    // every pass launches each kernel of the body once, those of the full
    // evaluation only when it is not a patch
    const long long patched = (long long)(hw_->patch[0] - patches_before);
    add_launches((graph_step_launches_ - graph_full_launches_) * out->brs +
                 graph_full_launches_ * (out->brs - patched));
    times_.evals += out->brs;
    times_.switches += out->brs + out->iters;
    if (rc) {   // the device error word was set: the state is not trusted
        val_ready_ = false;
        tour_valid_ = false;
        return rc;
    }
    val_ready_ = true;
    tour_valid_ = true;
    if (out->stop == GraphCtl::kEvalCap) return fail(PSI_ERR_LIMIT, "evaluation cap reached");
    if (out->stop == GraphCtl::kDeviceError) return fail(PSI_ERR_LIMIT, "graph solve loop stopped by a device error");
    if (out->stop != GraphCtl::kConverged) return fail(PSI_ERR_LIMIT, "graph solve loop stopped by its guard");
    return PSI_OK;
}

// solve_si as one graph launch; the same results and counts as solve().
int Solver::solve_graph(int32_t reset, int32_t *iters, int32_t *brs, int64_t max_evals)
{
    GraphCtl out;
    int rc = run_graph(reset != 0, max_evals, &out, nullptr);
    if (rc) return rc;
    *iters = out.iters;
    *brs = out.brs;
    return PSI_OK;
}

// A batch's solve_si loops as one graph launch: the union's loop ends when no
// game switches (a device-side decision, as for one game); every game's own
// counts come from its state in gstate_.  The same results and counts as
// the host-driven solve_batch.
int Solver::solve_batch_graph(std::vector<int4> &state)
{
    PSI_CUDA_TRY(cudaMemsetAsync(gstate_, 0, sizeof(int4) * (size_t)games_, stream_));
    PSI_CUDA_TRY(cudaMemsetAsync(gcount_, 0, sizeof(unsigned long long) * (size_t)games_, stream_));
    state.assign((size_t)games_, int4{});
    GraphCtl out;
    return run_graph(false, 0, &out, state.data());
}

}  // namespace psi
