// fyg_batch.cu -- uneven-length batches: many transforms of different lengths, packed back to
// back, run by one persistent kernel over a device work queue and launched as a CUDA graph.
// No counterpart in the reference, which runs one transform per dispatch call.
//
// Work decomposition: transforms of equal length form a group served by one plan (batch =
// multiplicity) whose user-buffer passes address the packed buffers through an offsets table.
// Every pass of every group is a descriptor (its PassParams); a work item is one tile of one
// descriptor.  Items are queued phase by phase (all first passes, then all second passes, ...),
// longest groups first within a phase.  A CTA pops items in order with an atomic counter; an
// item of pass p+1 waits until all tiles of pass p of its group are done.  Because items are
// popped in queue order and every popped item is held by a running CTA, the item it waits for
// is already being processed: the wait always ends.  It is still bounded (1 s by default): on
// expiry the kernel sets an error word and an abort flag, every CTA returns, and
// fyg_batch_status reports FYG_ERR_TIMEOUT.
#include <algorithm>
#include <cstdio>
#include <cstdlib>
#include <map>
#include <memory>
#include <mutex>
#include <numeric>
#include <string>
#include <vector>

#include "fyg_host.h"
#include "fyg_k_variant.cuh"

namespace fyg {

constexpr int kBatchThreads = 256;
constexpr int kBatchErrTimeout = 2;

struct BatchArgs {
    const PassParams* descs;
    const int2* items;
    int n_items;
    const int* need;         // tiles per descriptor
    const int* dep;          // descriptor each descriptor waits for (-1: none)
    int* done;               // completed tiles per descriptor
    int* head;               // queue head
    int* err;
    int* abort_flag;
    const void* user_in;
    void* user_out;
    const int64_t* offsets;  // element offset of every transform in the packed buffers
    unsigned long long timeout_ns;
};

__device__ __forceinline__ unsigned long long global_ns() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

template <int CLASS>
__global__ void __launch_bounds__(kBatchThreads) k_batch(const __grid_constant__ BatchArgs a) {
    extern __shared__ __align__(16) unsigned char smraw[];
    PassParams* sp = reinterpret_cast<PassParams*>(smraw);
    unsigned char* tsm = smraw + ((sizeof(PassParams) + 15) & ~(size_t)15);
    __shared__ int s_item, s_ok;
    for (;;) {
        if (threadIdx.x == 0) {
            int it = *reinterpret_cast<volatile int*>(a.abort_flag) ? a.n_items : atomicAdd(a.head, 1);
            if (it > a.n_items) it = a.n_items;
            int ok = 1;
            if (it < a.n_items) {
                const int dep = a.dep[a.items[it].x];
                if (dep >= 0) {
                    const int need = a.need[dep];
                    const unsigned long long t0 = global_ns();
                    while (atomicAdd(&a.done[dep], 0) < need) {
                        if (*reinterpret_cast<volatile int*>(a.abort_flag)) { ok = 0; break; }
                        if (global_ns() - t0 > a.timeout_ns) {
                            atomicOr(a.err, kBatchErrTimeout);
                            atomicExch(a.abort_flag, 1);
                            ok = 0;
                            break;
                        }
                        __nanosleep(200);
                    }
                    __threadfence();
                }
            }
            s_item = it;
            s_ok = ok;
        }
        __syncthreads();
        const int it = s_item;
        if (it >= a.n_items) break;
        if (s_ok) {
            const int2 d = a.items[it];
            const int4* src = reinterpret_cast<const int4*>(a.descs + d.x);
            int4* dst = reinterpret_cast<int4*>(sp);
            for (int w = threadIdx.x; w < (int)(sizeof(PassParams) / 16); w += blockDim.x) dst[w] = src[w];
            __syncthreads();
            if (threadIdx.x == 0) {
                if (sp->in_user) { sp->in = a.user_in; sp->in_offsets = a.offsets; }
                if (sp->out_user) { sp->out = a.user_out; sp->out_offsets = a.offsets; }
            }
            __syncthreads();
            if (sp->g.colmajor) tile_body<float, float, float, CLASS, true>(*sp, d.y, tsm);
            else tile_body<float, float, float, CLASS, false>(*sp, d.y, tsm);
            __syncthreads();
            if (threadIdx.x == 0) {
                __threadfence();
                atomicAdd(&a.done[d.x], 1);
            }
        }
        __syncthreads();
    }
}

template <int CLASS>
static cudaError_t launch_batch(const BatchArgs& a, size_t smem, cudaStream_t st, int* grid_out) {
    auto kern = k_batch<CLASS>;
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    int dev = 0, sms = 0, per_sm = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, kBatchThreads, smem);
    if (e != cudaSuccess) return e;
    int grid = std::max(1, sms * std::max(per_sm, 1));
    grid = std::min(grid, std::max(a.n_items, 1));
    *grid_out = grid;
    kern<<<grid, kBatchThreads, smem, st>>>(a);
    return cudaGetLastError();
}

}  // namespace fyg

using namespace fyg;

struct fyg_batch {
    std::vector<size_t> lengths;
    std::vector<int64_t> offsets;              // packed offsets (elements)
    int dtype = FYG_C32;
    int flags = 0;
    std::map<size_t, fyg_plan*> group_plans;   // per distinct length: batch = multiplicity
    std::map<size_t, std::vector<int>> members;
    std::map<size_t, fyg_plan*> single_plans;  // per distinct length: batch 1 (plain path)
    // persistent execution state (FP32 batches)
    bool persistent = false;
    int cls = 16;
    size_t smem = 0;
    int n_descs = 0, n_items = 0;
    DevBuf d_descs_fwd, d_descs_inv, d_items, d_need, d_dep, d_ids, d_offsets, d_state;
    std::vector<int> need_host;
    unsigned long long timeout_ns = 1000000000ull;
    // one instantiated graph per (direction, in, out, offsets)
    struct GraphKey {
        int dir; const void* in; void* out; const int64_t* off;
        bool operator<(const GraphKey& o) const {
            return std::tie(dir, in, out, off) < std::tie(o.dir, o.in, o.out, o.off);
        }
    };
    std::map<GraphKey, cudaGraphExec_t> graphs;
    cudaStream_t cap_stream = nullptr;
    int last_grid = 0;
    // branch form (FYG_FLAG_BATCH_BRANCHES): one regular plan per distinct length (batch =
    // multiplicity, register-resident kernels where they apply) whose passes address the packed
    // buffers through the offsets table; the plans run as parallel chains of one captured graph
    bool branches = false;
    std::map<size_t, fyg_plan*> branch_plans;
    std::map<size_t, int> branch_id0;          // first entry of the length's members in d_branch_ids
    DevBuf d_branch_ids;
    std::vector<cudaStream_t> branch_streams;
    std::vector<cudaEvent_t> branch_events;    // fork event, then one join event per stream
    // parallel chains of the graph: 32 measured best for the hybrid form (4096-length batch, split
    // at 4096: 2.34 ms; 128 chains: 2.76 ms, their kernels crowd out the persistent kernel)
    int max_branches = 32;

    int* done_ptr() { return reinterpret_cast<int*>(d_state.ptr); }
    int* head_ptr() { return done_ptr() + n_descs; }
    int* err_ptr() { return head_ptr() + 1; }
    int* abort_ptr() { return head_ptr() + 2; }

    ~fyg_batch() {
        for (auto& kv : graphs) cudaGraphExecDestroy(kv.second);
        if (cap_stream) cudaStreamDestroy(cap_stream);
        for (cudaStream_t s : branch_streams) cudaStreamDestroy(s);
        for (cudaEvent_t e : branch_events) cudaEventDestroy(e);
        for (auto& kv : branch_plans) fyg_plan_destroy(kv.second);
        for (auto& kv : group_plans) fyg_plan_destroy(kv.second);
        for (auto& kv : single_plans) fyg_plan_destroy(kv.second);
    }
};

namespace {

// Builds the descriptor tables and the work queue for one direction set (forward and inverse
// share items, need and dep; only the PassParams differ).
int build_persistent(fyg_batch* b) {
    std::vector<PassParams> fwd, inv;
    std::vector<int> need, dep, ids, fwd_id0, inv_id0;
    struct G { size_t len; int first_desc; int npass; double work; };
    std::vector<G> groups;
    size_t smem = 0;
    int cls = 16;
    for (auto& kv : b->group_plans) {
        const size_t len = kv.first;
        fyg_plan* pl = kv.second;
        if (pl->strategy == GS_COPY || pl->strategy == GS_SPLIT || pl->chunk != pl->batch || pl->compute_bytes != 8)
            return FYG_ERR_UNSUPPORTED;
        const std::vector<int>& mem = b->members[len];
        const int id0 = (int)ids.size();
        ids.insert(ids.end(), mem.begin(), mem.end());
        G g{len, (int)fwd.size(), (int)pl->fwd.size(), (double)len * mem.size()};
        for (int dirn = 0; dirn < 2; ++dirn) {
            const std::vector<PassDesc>& pipe = dirn == 0 ? pl->fwd : pl->inv;
            for (size_t i = 0; i < pipe.size(); ++i) {
                const PassDesc& d = pipe[i];
                PassParams p = d.p;
                p.ncols = (int64_t)pl->batch * p.Rr;
                p.x0buf = pl->x0buf.ptr;
                p.dcbuf = pl->dcbuf.ptr;
                p.in_user = d.in_role == ROLE_IN;
                p.out_user = d.out_role == ROLE_OUT;
                p.in = d.in_role == ROLE_S0 ? pl->scratch0.ptr : d.in_role == ROLE_S1 ? pl->scratch1.ptr : nullptr;
                p.out = d.out_role == ROLE_S0 ? pl->scratch0.ptr : d.out_role == ROLE_S1 ? pl->scratch1.ptr : nullptr;
                p.in_offsets = p.out_offsets = nullptr;
                p.ids = nullptr;   // set once the id table is on the device
                if (dirn == 0) {
                    fwd.push_back(p);
                    fwd_id0.push_back(id0);
                    need.push_back((int)((p.ncols + p.g.C - 1) / p.g.C));
                    dep.push_back(i == 0 ? -1 : (int)fwd.size() - 2);
                    smem = std::max(smem, d.smem);
                    if (d.kv == KV_F32_C32) cls = 32;
                } else {
                    inv.push_back(p);
                    inv_id0.push_back(id0);
                }
            }
        }
        groups.push_back(g);
    }
    int rc = b->d_ids.upload(ids.data(), std::max<size_t>(ids.size(), 1) * sizeof(int));
    if (rc) return rc;
    for (size_t i = 0; i < fwd.size(); ++i) fwd[i].ids = reinterpret_cast<const int*>(b->d_ids.ptr) + fwd_id0[i];
    for (size_t i = 0; i < inv.size(); ++i) inv[i].ids = reinterpret_cast<const int*>(b->d_ids.ptr) + inv_id0[i];
    // queue: phase by phase, longest groups first
    std::vector<int> order(groups.size());
    std::iota(order.begin(), order.end(), 0);
    std::sort(order.begin(), order.end(), [&](int x, int y) { return groups[x].work > groups[y].work; });
    int maxp = 0;
    for (auto& g : groups) maxp = std::max(maxp, g.npass);
    std::vector<int2> items;
    for (int ph = 0; ph < maxp; ++ph)
        for (int gi : order) {
            const G& g = groups[gi];
            if (ph >= g.npass) continue;
            const int desc = g.first_desc + ph;
            for (int t = 0; t < need[desc]; ++t) items.push_back(make_int2(desc, t));
        }
    b->n_descs = (int)fwd.size();
    b->n_items = (int)items.size();
    b->need_host = need;
    b->smem = ((sizeof(PassParams) + 15) & ~(size_t)15) + smem;
    b->cls = cls;
    if (b->smem > 232448) return set_error(FYG_ERR_UNSUPPORTED, "batch tile exceeds shared memory");
    rc = b->d_descs_fwd.upload(fwd.data(), fwd.size() * sizeof(PassParams));
    if (!rc) rc = b->d_descs_inv.upload(inv.data(), inv.size() * sizeof(PassParams));
    if (!rc) rc = b->d_items.upload(items.data(), std::max<size_t>(items.size(), 1) * sizeof(int2));
    if (!rc) rc = b->d_need.upload(need.data(), need.size() * sizeof(int));
    if (!rc) rc = b->d_dep.upload(dep.data(), dep.size() * sizeof(int));
    if (!rc) rc = b->d_offsets.upload(b->offsets.data(), b->offsets.size() * sizeof(int64_t));
    if (!rc) rc = b->d_state.alloc((b->n_descs + 4) * sizeof(int));
    return rc;
}

int launch_persistent(fyg_batch* b, const void* in, void* out, const int64_t* offs, int direction,
                      cudaStream_t st) {
    BatchArgs a;
    a.descs = reinterpret_cast<const PassParams*>(direction == FYG_INVERSE ? b->d_descs_inv.ptr : b->d_descs_fwd.ptr);
    a.items = reinterpret_cast<const int2*>(b->d_items.ptr);
    a.n_items = b->n_items;
    a.need = reinterpret_cast<const int*>(b->d_need.ptr);
    a.dep = reinterpret_cast<const int*>(b->d_dep.ptr);
    a.done = b->done_ptr();
    a.head = b->head_ptr();
    a.err = b->err_ptr();
    a.abort_flag = b->abort_ptr();
    a.user_in = in;
    a.user_out = out;
    a.offsets = offs ? offs : reinterpret_cast<const int64_t*>(b->d_offsets.ptr);
    a.timeout_ns = b->timeout_ns;
    cudaError_t e = cudaMemsetAsync(b->d_state.ptr, 0, (b->n_descs + 4) * sizeof(int), st);
    if (e != cudaSuccess) return cuda_error(e, "batch state reset");
    e = b->cls > 16 ? launch_batch<32>(a, b->smem, st, &b->last_grid) : launch_batch<16>(a, b->smem, st, &b->last_grid);
    if (e != cudaSuccess) return cuda_error(e, "persistent batch launch");
    return FYG_OK;
}

}  // namespace

namespace {

// Autotune cache key of a batch: element type and an FNV-1a hash of the length sequence.
std::string batch_key(const size_t* lengths, size_t count, int dtype) {
    uint64_t h = 1469598103934665603ull;
    auto mix = [&](uint64_t v) {
        for (int i = 0; i < 8; ++i) {
            h ^= (v >> (8 * i)) & 0xff;
            h *= 1099511628211ull;
        }
    };
    mix((uint64_t)count);
    for (size_t i = 0; i < count; ++i) mix((uint64_t)lengths[i]);
    char buf[64];
    std::snprintf(buf, sizeof(buf), "batch%s:%zu:%016llx", dtype == FYG_C32 ? "32" : "64", count,
                  (unsigned long long)h);
    return buf;
}

// The batch autotuner's candidate, used by fyg_batch_create in place of a cache entry while set.
thread_local const TuneChoice* g_candidate = nullptr;

// Sets the group-plan options for this thread while alive.
struct BatchOptions {
    BatchOptions(int radix_cap, int single_kb) { set_batch_tile_options(radix_cap, (size_t)single_kb << 10); }
    ~BatchOptions() { set_batch_tile_options(0, 0); }
};

}  // namespace

namespace {

// The branch form: every distinct length's plan is a chain of kernels on one of up to 32 streams
// forked from the capture stream (lengths with the most work first, each to the least loaded
// stream), joined back, captured once per (direction, buffers, offsets) and replayed.
int capture_branches(fyg_batch* b, const void* in, void* out, const int64_t* offs, int direction,
                     cudaStream_t cap) {
    const size_t eb = b->dtype == FYG_C32 ? 8 : 16;
    const int nb = (int)std::min<size_t>((size_t)b->max_branches, b->branch_plans.size());
    while ((int)b->branch_streams.size() < nb) {
        cudaStream_t s;
        cudaError_t e = cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking);
        if (e != cudaSuccess) return cuda_error(e, "branch stream");
        b->branch_streams.push_back(s);
    }
    while ((int)b->branch_events.size() < nb + 1) {
        cudaEvent_t ev;
        cudaError_t e = cudaEventCreateWithFlags(&ev, cudaEventDisableTiming);
        if (e != cudaSuccess) return cuda_error(e, "branch event");
        b->branch_events.push_back(ev);
    }
    cudaError_t e = cudaEventRecord(b->branch_events[0], cap);
    for (int k = 0; k < nb && e == cudaSuccess; ++k) e = cudaStreamWaitEvent(b->branch_streams[k], b->branch_events[0], 0);
    if (e != cudaSuccess) return cuda_error(e, "branch fork");
    std::vector<std::pair<double, size_t>> work;
    for (auto& kv : b->members) {
        if (!b->branch_plans.count(kv.first)) continue;   // in the persistent kernel
        const double n = (double)kv.first;
        work.push_back({n * std::max(1.0, std::log2(n)) * (double)kv.second.size(), kv.first});
    }
    std::sort(work.rbegin(), work.rend());
    std::vector<double> load(nb, 0.0);
    const int* ids = reinterpret_cast<const int*>(b->d_branch_ids.ptr);
    for (auto& w : work) {
        const int k = (int)(std::min_element(load.begin(), load.end()) - load.begin());
        load[k] += w.first;
        const cudaStream_t s = b->branch_streams[k];
        fyg_plan* pl = b->branch_plans[w.second];
        if (pl->strategy == GS_COPY) {
            // length 1: the identity, one element per member (host offsets)
            for (int m : b->members[w.second]) {
                const int64_t o = b->offsets[m];
                e = cudaMemcpyAsync((char*)out + o * eb, (const char*)in + o * eb, eb, cudaMemcpyDeviceToDevice, s);
                if (e != cudaSuccess) return cuda_error(e, "length-1 copy");
            }
            continue;
        }
        const int rc = run_plan_offsets(pl, in, out, offs, ids + b->branch_id0[w.second], direction, s);
        if (rc) return rc;
    }
    // the persistent kernel (shorter lengths) on the capture stream, alongside the branches
    if (b->persistent) {
        const int rc = launch_persistent(b, in, out, offs == reinterpret_cast<const int64_t*>(b->d_offsets.ptr) ? nullptr : offs,
                                         direction, cap);
        if (rc) return rc;
    }
    for (int k = 0; k < nb && e == cudaSuccess; ++k) {
        e = cudaEventRecord(b->branch_events[k + 1], b->branch_streams[k]);
        if (e == cudaSuccess) e = cudaStreamWaitEvent(cap, b->branch_events[k + 1], 0);
    }
    return e == cudaSuccess ? FYG_OK : cuda_error(e, "branch join");
}

}  // namespace

static int execute_branches(fyg_batch* b, const void* in, void* out, const int64_t* offsets_dev, int direction,
                            cudaStream_t st) {
    const int64_t* offs = offsets_dev ? offsets_dev : reinterpret_cast<const int64_t*>(b->d_offsets.ptr);
    fyg_batch::GraphKey key{direction, in, out, offsets_dev};
    auto it = b->graphs.find(key);
    if (it == b->graphs.end()) {
        if (!b->cap_stream) {
            cudaError_t e = cudaStreamCreateWithFlags(&b->cap_stream, cudaStreamNonBlocking);
            if (e != cudaSuccess) return cuda_error(e, "capture stream");
        }
        cudaError_t e = cudaStreamBeginCapture(b->cap_stream, cudaStreamCaptureModeThreadLocal);
        if (e != cudaSuccess) return cuda_error(e, "begin capture");
        int rc = capture_branches(b, in, out, offs, direction, b->cap_stream);
        cudaGraph_t g = nullptr;
        e = cudaStreamEndCapture(b->cap_stream, &g);
        if (rc) { if (g) cudaGraphDestroy(g); return rc; }
        if (e != cudaSuccess) return cuda_error(e, "end capture");
        cudaGraphExec_t ex = nullptr;
        e = cudaGraphInstantiate(&ex, g, 0);
        cudaGraphDestroy(g);
        if (e != cudaSuccess) return cuda_error(e, "graph instantiate");
        it = b->graphs.emplace(key, ex).first;
    }
    const cudaError_t e = cudaGraphLaunch(it->second, st);
    return e == cudaSuccess ? FYG_OK : cuda_error(e, "graph launch");
}

extern "C" {

int fyg_batch_create_ex(const size_t* lengths, size_t count, int dtype, int flags, int form, size_t split,
                        int radix_cap, int single_tile_kb, fyg_batch** out) {
    if (form < 0 || form > 2) return set_error(FYG_ERR_INVALID_ARG, "form must be 0, 1 or 2");
    TuneChoice cc;
    cc.max_pass_radix = (uint64_t)std::max(radix_cap, 0);
    cc.cols = std::max(single_tile_kb, 0);
    cc.order = form;
    cc.conv_length = (uint64_t)split;
    g_candidate = &cc;
    const int rc = fyg_batch_create(lengths, count, dtype, flags | FYG_FLAG_AUTOTUNED, out);
    g_candidate = nullptr;
    return rc;
}

int fyg_batch_create(const size_t* lengths, size_t count, int dtype, int flags, fyg_batch** out) {
    clear_error();
    if (!out || (!lengths && count)) return set_error(FYG_ERR_NULL_PTR, "null argument");
    *out = nullptr;
    if (dtype != FYG_C32 && dtype != FYG_C64) return set_error(FYG_ERR_INVALID_ARG, "bad dtype");
    TuneChoice tc;
    if (flags & FYG_FLAG_AUTOTUNED) {
        if (g_candidate) tc = *g_candidate;
        else if (!tune_lookup_key(batch_key(lengths, count, dtype), &tc)) tc = TuneChoice();
    }
    // lengths above `split` run in the branch form, the others in the persistent kernel:
    // SIZE_MAX by default, 0 with FYG_FLAG_BATCH_BRANCHES, else the tuner's choice (order 1:
    // all branches, order 2: the split stored in conv_length); FP64 batches have no persistent
    // kernel and run in the branch form
    size_t split = SIZE_MAX;
    if ((flags & FYG_FLAG_AUTOTUNED) && tc.order == 1) split = 0;
    if ((flags & FYG_FLAG_AUTOTUNED) && tc.order == 2) split = (size_t)tc.conv_length;
    if ((flags & FYG_FLAG_BATCH_BRANCHES) || dtype != FYG_C32) split = 0;
    flags &= ~(FYG_FLAG_AUTOTUNED | FYG_FLAG_BATCH_BRANCHES);
    BatchOptions opts((int)tc.max_pass_radix, tc.cols);
    auto b = std::make_unique<fyg_batch>();
    b->dtype = dtype;
    b->flags = flags;
    int64_t off = 0;
    for (size_t i = 0; i < count; ++i) {
        if (lengths[i] < 1) return set_error(FYG_ERR_INVALID_LENGTH, "length must be >= 1");
        b->lengths.push_back(lengths[i]);
        b->offsets.push_back(off);
        b->members[lengths[i]].push_back((int)i);
        off += (int64_t)lengths[i];
    }
    for (auto& kv : b->members) {
        if (kv.first <= split) {
            fyg_plan* p = nullptr;
            int rc = fyg_plan_create(kv.first, dtype, kv.second.size(),
                                     flags | FYG_FLAG_NO_L2_CHUNK | FYG_FLAG_SMALL_TILES, &p);
            if (rc) return rc;
            b->group_plans[kv.first] = p;
        }
    }
    if (!b->group_plans.empty()) {
        int rc = build_persistent(b.get());
        if (rc == FYG_OK) b->persistent = true;
        else if (rc != FYG_ERR_UNSUPPORTED) return rc;
        clear_error();
        if (!b->persistent) {   // no persistent kernel for these plans: they join the branch form
            for (auto& kv : b->group_plans) fyg_plan_destroy(kv.second);
            b->group_plans.clear();
            split = 0;
        }
    }
    std::vector<int> ids;
    for (auto& kv : b->members) {
        if (kv.first <= split) continue;
        fyg_plan* p = nullptr;
        int rc = fyg_plan_create(kv.first, dtype, kv.second.size(), flags | FYG_FLAG_NO_L2_CHUNK, &p);
        if (rc) return rc;
        b->branch_plans[kv.first] = p;
        b->branch_id0[kv.first] = (int)ids.size();
        ids.insert(ids.end(), kv.second.begin(), kv.second.end());
    }
    if (!b->branch_plans.empty()) {
        b->branches = true;
        int rc = b->d_branch_ids.upload(ids.data(), ids.size() * sizeof(int));
        if (!rc && !b->persistent)
            rc = b->d_offsets.upload(b->offsets.data(), std::max<size_t>(b->offsets.size(), 1) * sizeof(int64_t));
        if (rc) return rc;
    }
    *out = b.release();
    return FYG_OK;
}

int fyg_batch_destroy(fyg_batch* batch) {
    delete batch;
    return FYG_OK;
}

int fyg_batch_execute_plain(fyg_batch* b, const void* in, void* out, int direction, void* stream) {
    clear_error();
    if (!b || !in || !out) return set_error(FYG_ERR_NULL_PTR, "null argument");
    const size_t eb = b->dtype == FYG_C32 ? 8 : 16;
    // one plan per distinct length with batch 1, created on first use
    for (size_t len : b->lengths) {
        if (b->single_plans.count(len)) continue;
        fyg_plan* p = nullptr;
        const int rc = fyg_plan_create(len, b->dtype, 1, b->flags, &p);
        if (rc) return rc;
        b->single_plans[len] = p;
    }
    for (size_t i = 0; i < b->lengths.size(); ++i) {
        const char* x = (const char*)in + b->offsets[i] * eb;
        char* y = (char*)out + b->offsets[i] * eb;
        int rc = fyg_execute(b->single_plans[b->lengths[i]], x, y, direction, stream);
        if (rc) return rc;
    }
    return FYG_OK;
}

int fyg_batch_execute(fyg_batch* b, const void* in, void* out, const int64_t* offsets_dev, int direction,
                      void* stream) {
    clear_error();
    if (!b || !in || !out) return set_error(FYG_ERR_NULL_PTR, "null argument");
    if (direction != FYG_FORWARD && direction != FYG_INVERSE)
        return set_error(FYG_ERR_INVALID_ARG, "direction must be FYG_FORWARD or FYG_INVERSE");
    if (b->lengths.empty()) return FYG_OK;
    const cudaStream_t st = (cudaStream_t)stream;
    if (b->branches) return execute_branches(b, in, out, offsets_dev, direction, st);
    if (!b->persistent) return set_error(FYG_ERR_UNSUPPORTED, "batch has no execution form");
    fyg_batch::GraphKey key{direction, in, out, offsets_dev};
    auto it = b->graphs.find(key);
    if (it == b->graphs.end()) {
        if (!b->cap_stream) {
            cudaError_t e = cudaStreamCreateWithFlags(&b->cap_stream, cudaStreamNonBlocking);
            if (e != cudaSuccess) return cuda_error(e, "capture stream");
        }
        cudaError_t e = cudaStreamBeginCapture(b->cap_stream, cudaStreamCaptureModeThreadLocal);
        if (e != cudaSuccess) return cuda_error(e, "begin capture");
        int rc = launch_persistent(b, in, out, offsets_dev, direction, b->cap_stream);
        cudaGraph_t g = nullptr;
        e = cudaStreamEndCapture(b->cap_stream, &g);
        if (rc) { if (g) cudaGraphDestroy(g); return rc; }
        if (e != cudaSuccess) return cuda_error(e, "end capture");
        cudaGraphExec_t ex = nullptr;
        e = cudaGraphInstantiate(&ex, g, 0);
        cudaGraphDestroy(g);
        if (e != cudaSuccess) return cuda_error(e, "graph instantiate");
        it = b->graphs.emplace(key, ex).first;
    }
    cudaError_t e = cudaGraphLaunch(it->second, st);
    if (e != cudaSuccess) return cuda_error(e, "graph launch");
    return FYG_OK;
}

int fyg_batch_status(fyg_batch* b, void* stream) {
    clear_error();
    if (!b) return set_error(FYG_ERR_NULL_PTR, "null batch");
    if (b->branches) {
        // the device error bits of every branch length's plan
        for (auto& kv : b->branch_plans) {
            int st = 0;
            const int rc = fyg_plan_status(kv.second, stream, &st);
            if (rc) return rc;
            if (st) return set_error(FYG_ERR_CUDA, "kernel error bits " + std::to_string(st) + " (length " +
                                                       std::to_string(kv.first) + ")");
        }
    }
    if (!b->persistent) return FYG_OK;
    cudaError_t e = cudaStreamSynchronize((cudaStream_t)stream);
    if (e != cudaSuccess) return cuda_error(e, "stream synchronize");
    int err = 0;
    e = cudaMemcpy(&err, b->err_ptr(), sizeof(int), cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) return cuda_error(e, "status read");
    if (err & kBatchErrTimeout)
        return set_error(FYG_ERR_TIMEOUT, "a work item waited longer than the batch's limit for its dependency");
    return FYG_OK;
}

int fyg_batch_inject_stall(fyg_batch* b, int enable, int timeout_ms) {
    clear_error();
    if (!b) return set_error(FYG_ERR_NULL_PTR, "null batch");
    if (!b->persistent) return set_error(FYG_ERR_UNSUPPORTED, "batch has no persistent path");
    std::vector<int> need = b->need_host;
    if (enable) {
        // the first descriptor another one waits for: its completion count becomes unreachable
        std::vector<int> dep(b->n_descs);
        cudaError_t e = cudaMemcpy(dep.data(), b->d_dep.ptr, dep.size() * sizeof(int), cudaMemcpyDeviceToHost);
        if (e != cudaSuccess) return cuda_error(e, "dep read");
        int victim = -1;
        for (int d : dep) if (d >= 0) { victim = d; break; }
        if (victim < 0) return set_error(FYG_ERR_UNSUPPORTED, "no multi-pass group to stall");
        need[victim] = 1 << 30;
    }
    b->timeout_ns = enable ? (unsigned long long)std::max(timeout_ms, 1) * 1000000ull : 1000000000ull;
    for (auto& kv : b->graphs) cudaGraphExecDestroy(kv.second);
    b->graphs.clear();
    cudaError_t e = cudaMemcpy(b->d_need.ptr, need.data(), need.size() * sizeof(int), cudaMemcpyHostToDevice);
    if (e != cudaSuccess) return cuda_error(e, "need upload");
    return FYG_OK;
}

}  // extern "C"

// Times the persistent launch of this length sequence under each group-plan option set (stage
// radix cap 16 or 32, single-pass tile cap 48 / 100 / 160 KB of shared memory) on random data
// and caches the fastest; fyg_batch_create(..., FYG_FLAG_AUTOTUNED) uses it.
extern "C" int fyg_batch_autotune(const size_t* lengths, size_t count, int dtype, const char* cache_path,
                                  double* best_ms) {
    clear_error();
    if (!lengths || count == 0) return set_error(FYG_ERR_NULL_PTR, "no lengths");
    if (dtype != FYG_C32) return set_error(FYG_ERR_UNSUPPORTED, "batch autotuning needs FYG_C32 (persistent kernel)");
    size_t total = 0;
    for (size_t i = 0; i < count; ++i) total += lengths[i];
    DevBuf in, out;
    int rc = in.alloc(total * 8);
    if (!rc) rc = out.alloc(total * 8);
    if (!rc) rc = fyg_fill_random_device(11, 1, dtype, total, in.ptr, nullptr);
    if (rc) return rc;
    const bool verbose = std::getenv("FYG_AUTOTUNE_VERBOSE") != nullptr;
    // {stage radix cap, single-pass tile KB, form, split}: form 0 persistent kernel, 1 branches,
    // 2 lengths up to `split` in the persistent kernel and the longer ones in branches
    const int cand[][4] = {{16, 100, 0, 0}, {32, 100, 0, 0}, {16, 48, 0, 0}, {32, 160, 0, 0}, {0, 0, 1, 0},
                           {16, 100, 2, 4096}, {16, 100, 2, 16384}, {32, 100, 2, 4096}};
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    TuneChoice best;
    bool have = false;
    for (const auto& c : cand) {
        fyg_batch* b = nullptr;
        const bool br = c[2] == 1;
        if (fyg_batch_create_ex(lengths, count, dtype, 0, c[2], (size_t)c[3], c[0], c[1], &b) != FYG_OK) continue;
        double t = 1e30;
        (void)br;
        bool ok = (b->persistent || b->branches) &&
                  fyg_batch_execute(b, in.ptr, out.ptr, nullptr, FYG_FORWARD, nullptr) == FYG_OK;
        for (int rep = 0; rep < 3 && ok; ++rep) {
            cudaEventRecord(e0, nullptr);
            ok = fyg_batch_execute(b, in.ptr, out.ptr, nullptr, FYG_FORWARD, nullptr) == FYG_OK;
            cudaEventRecord(e1, nullptr);
            ok = ok && cudaEventSynchronize(e1) == cudaSuccess && fyg_batch_status(b, nullptr) == FYG_OK;
            float ms = 0;
            cudaEventElapsedTime(&ms, e0, e1);
            t = std::min(t, (double)ms);
        }
        fyg_batch_destroy(b);
        if (verbose)
            std::fprintf(stderr, "fyg_batch_autotune form=%d split=%d radix_cap=%d single_tile_kb=%d: %s %.4f ms\n",
                         c[2], c[3], c[0], c[1], ok ? "ok" : "failed", ok ? t : 0.0);
        if (ok && (!have || t < best.ms)) {
            best = TuneChoice();
            best.max_pass_radix = (uint64_t)c[0];
            best.cols = c[1];
            best.order = c[2];
            best.conv_length = (uint64_t)c[3];
            best.ms = t;
            have = true;
        }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    clear_error();
    if (!have) return set_error(FYG_ERR_UNSUPPORTED, "batch autotune: no candidate ran");
    if (best_ms) *best_ms = best.ms;
    return tune_store_key(batch_key(lengths, count, dtype), best, cache_path);
}
