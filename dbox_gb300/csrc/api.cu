// C ABI of libdbox_gpu.so (declared in include/dbox_gpu.h).
//
// Host side: world creation (the reference's b2World.CreateBody /
// b2Body.CreateFixture / b2World.CreateJoint bookkeeping), upload of the
// structure-of-arrays batch to the GPU, step launches (plain or replayed from a
// CUDA graph) and state export/import.  All per-step work runs in the kernels
// of step.cu; this file only moves data and launches.
#include <cuda_runtime.h>
#include <cfloat>
#include <stdint.h>
#include <string.h>
#include <stdio.h>
#include <stdarg.h>
#include <string>
#include <unordered_map>
#include <vector>
#include <algorithm>
#include <mutex>

#include "world.cuh"
#include "host_geom.h"

extern "C" int dbox_launch_step(const dg::Ctx* x, cudaStream_t stream, int* launches);
extern "C" const void* dbox_solve_kernel();
extern "C" const void* dbox_step_fused_kernel();
extern "C" int dbox_launch_steps_fused(const dg::Ctx* x, cudaStream_t stream, int* launches);
extern "C" int dbox_big_solve_init(int* cluster);
const dg::MlpDev* dbox_mlp_device_view(const dbox_mlp* m, dg::MlpDev* out);
extern "C" int dbox_launch_step_ev(const dg::Ctx* x, cudaStream_t stream, int* launches, cudaEvent_t* ev);
extern "C" int dbox_launch_collide(const dg::Ctx* x, cudaStream_t stream);
extern "C" int dbox_launch_solve(const dg::Ctx* x, cudaStream_t stream, int* launches);
extern "C" int dbox_launch_gather_transforms(int n, const dbox_body_state* bs, float* out, cudaStream_t s);
extern "C" int dbox_launch_apply_forces(int n, dbox_body_state* bs, const float* f, cudaStream_t s);
extern "C" int dbox_launch_query_build(const dbox_query_buffers* b, cudaStream_t s);
extern "C" int dbox_launch_query_aabb(const dbox_query_buffers* b, int n, const int* world, const dbox_aabb* boxes,
                                      int cap, int* counts, int* out, cudaStream_t s);
extern "C" int dbox_launch_raycast(const dbox_query_buffers* b, int n, const int* world, const dbox_vec2* p1,
                                   const dbox_vec2* p2, int mode, int cap, int* counts, dbox_ray_hit* out,
                                   cudaStream_t s);
extern "C" int dbox_query_warps_per_block();
extern "C" int dbox_launch_collide_pairs(int n, const dg::DFixture* fa, const float4* xa, const dg::DFixture* fb,
                                         const float4* xb, dbox_contact_state* out, cudaStream_t stream);

namespace {

thread_local std::string g_last_error = "";

int fail(int code, const char* fmt, ...) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    g_last_error = buf;
    return code;
}

}  // namespace

// error text for the other translation units of the library (not part of the public header)
extern "C" int dbox_set_error(int code, const char* msg) { return fail(code, "%s", msg); }

namespace {

#define CU(call)                                                                          \
    do {                                                                                  \
        cudaError_t e_ = (call);                                                          \
        if (e_ != cudaSuccess) return fail(DBOX_ERR_CUDA, "%s: %s", #call, cudaGetErrorString(e_)); \
    } while (0)

// A b2ChainShape as created (b2chainshape.d:45-110): its vertex list (a loop repeats the first
// vertex), ghost vertices and the definition's density; its child edges are the fixtures
// [first, first + vertices - 1).
struct ChainRec {
    std::vector<dbox_vec2> v;
    dbox_vec2 prev, next;
    int has_prev, has_next;
    float density;
    int first;
    int dead;
};

// b2DynamicTree node allocation as far as proxy ids depend on it (b2dynamictree.d:110-134,
// 516-564): freed nodes are reused last in, first out, before never-used ones.  A new proxy
// takes a leaf and then, unless the tree was empty, an internal parent; destroying a proxy
// frees its parent (unless it was the root) and then the leaf.  So the stack always holds
// (leaf, parent) pairs, with one lone leaf on top while the tree is empty: a parent's id is
// never handed out as a proxy id, and its place in the stack is all that is kept (-1).  Moving
// a proxy frees and at once retakes its parent, which changes nothing here.
struct ProxyIds {
    std::vector<int> free_nodes;
    int fresh = 0;      // lowest node id never used
    int live = 0;       // proxies in the tree
    int take() {
        if (free_nodes.empty()) return fresh++;
        int id = free_nodes.back();
        free_nodes.pop_back();
        return id;
    }
    int create() {
        int id = take();
        if (live > 0) take();                                           // the new leaf's parent
        ++live;
        return id;
    }
    void destroy(int id) {
        if (live > 1) free_nodes.push_back(-1);                         // RemoveLeaf frees the parent first
        free_nodes.push_back(id);
        --live;
    }
};

// worlds with at least this many fixtures generate their end-of-Solve pairs on a block of
// 1024 threads instead of their solve warp
constexpr int kPairBlockFixtures = 4096;

struct HostWorld {
    std::vector<ChainRec> chains;
    ProxyIds ids;
    std::vector<char> body_dead;   // destroyed bodies (kept as all-zero records so indices stay put)
    std::vector<dbox_body_state> bs;
    std::vector<dg::BodyStatic> bst;
    std::vector<std::vector<int>> body_fix;     // fixture indices per body, newest first
    std::vector<dg::DFixture> fx;
    std::vector<dbox_proxy_state> px;
    std::vector<dg::DJoint> jt;
    std::vector<dbox_contact_state> ct;
    dg::WorldDyn wd;
    HostWorld() { memset(&wd, 0, sizeof(wd)); wd.flags = 4u; wd.step_complete = 1; }
};

template <class T> struct DBuf {
    T* p = nullptr;
    size_t n = 0;
    int alloc(size_t count) {
        free();
        n = count;
        if (count == 0) count = 1;
        if (cudaMalloc(&p, count * sizeof(T)) != cudaSuccess) { p = nullptr; return -1; }
        return 0;
    }
    void free() { if (p) cudaFree(p); p = nullptr; n = 0; }
};

}  // namespace

struct dbox_world {
    std::vector<HostWorld> worlds;
    float2 gravity;
    int warm = 1, continuous = 1, substep = 0, allow_sleep = 1, autoclear = 1;
    dbox_world_caps caps;
    bool on_device = false;     // device holds the authoritative dynamic state
    bool mirrors_fresh = false; // host mirrors equal the device state (no device work since the last download)
    bool dirty = true;          // host structure changed since the last upload
    cudaStream_t stream = nullptr;
    // device arrays
    DBuf<dg::WorldInfo> d_wi;
    DBuf<dg::WorldDyn> d_wd;
    DBuf<dbox_body_state> d_bs;
    DBuf<dg::BodyStatic> d_bst;
    DBuf<int> d_body_fix, d_jadj_joint, d_jadj_other;
    DBuf<dg::DFixture> d_fx;
    DBuf<dbox_proxy_state> d_px;
    DBuf<dg::DJoint> d_jt;
    DBuf<dbox_contact_state> d_ct;
    DBuf<int> d_cworld;
    DBuf<unsigned long long> d_hash;
    DBuf<int2> d_pairs;
    DBuf<int> s_woken, s_adj_start, s_cursor, s_stack, s_isl_body, s_body_island, s_last, s_isl_bstart,
        s_isl_cstart, s_isl_jstart, s_isl_flags, s_pcount, s_moved, s_cstate, s_isl_contact, s_level, s_lcur, s_tcand,
        s_sched_v, s_lvl_v, s_sched_p, s_lvl_p, s_tmp, s_isl_joint, s_accept, g_status;
    DBuf<unsigned> s_isl_minsep, s_isl_sleep;
    DBuf<dg::VRow> d_vr, d_tvr;
    DBuf<dg::PRow> d_pr, d_tpr;
    DBuf<int> s_vpos, d_solve_world, d_solve_smem;
    int solve_blocks = 0, solve_smem_floats = 0;
    int solve_wpb = dg::kSolveWarps;    // warp slots (worlds) per block of the solve kernel
    int solve_budget = 0;               // body budget per block (0: chosen from the worlds)
    int solve_isolate = 0;              // this many largest worlds get a block of their own
    // world-queue mapping: a resident wave of warps takes worlds costliest first
    int solve_queue_mode = 0;           // 1: queue mapping, 0: packing into blocks
    int solve_heavy = 0;                // costliest worlds spread one per SM sub-partition
    int solve_exclusive = 0;            // their sub-partitions take no other world meanwhile
    int solve_bps = 0;                  // resident blocks per SM of the queue mapping (0: as many as fit)
    int solve_cap = 0;
    int nsm = 0;
    DBuf<int> d_solve_order, d_solve_queue;
    std::vector<float> world_cost;      // per world, for the queue order (empty: body counts)
    DBuf<dg::SweepSnap> d_snap;
    DBuf<float> d_io;           // staging for bulk force upload / transform readback (3 floats per body)
    DBuf<int2> s_cbody, s_adj_items, s_isl_pair;
    DBuf<unsigned char> s_cq, s_cvis, s_bfl;
    DBuf<float> s_sbody;
    DBuf<unsigned long long> d_prof;
    int profiling = 0;
    // learned warm start and solver-quality measurement
    int ws_mode = 0;
    dbox_mlp* mlp = nullptr;
    int sample_cap = 0;
    DBuf<float> d_samples, s_feat, s_vsave;
    DBuf<unsigned> d_sample_count;
    DBuf<int> s_slog, s_pend;
    int measure = 0;
    int wait_polls = 1 << 20;   // budget of one mbarrier wait in the solve kernel (polls)
    int island_solver = 0;      // 0: a large world's Solve on a block (k_solve_big), 1: on a warp
    int big_cluster = 1;        // blocks of k_solve_big's cluster per large world (its level sweeps)
    int fused_step = 0;         // 1: whole steps in one launch (k_step_fused) where the handle allows
    // contact listener
    DBuf<dbox_contact_event> d_events;
    DBuf<unsigned> s_sapk0, s_sapk1;
    DBuf<int> s_sapi0, s_sapi1;
    DBuf<float4> s_sapbox;
    DBuf<int> d_porder;         // per world: fixtures in proxy-id order
    DBuf<int> s_sapcell;        // per world: the broad-phase grid's cell tables
    DBuf<int> d_big;            // worlds whose end-of-Solve pairs a block generates
    int n_big = 0;
    DBuf<unsigned char> s_cevt;
    std::vector<dbox_contact_event> h_events;
    std::vector<dg::WorldInfo> wi;
    int total_bodies = 0, total_fixtures = 0, total_contacts = 0, total_joints = 0;
    // graph replay
    cudaGraphExec_t graph = nullptr;
    float g_dt = -1.0f;
    int g_vi = -1, g_pi = -1;
    int graph_flags = -1;
    int g_launches = 0;                 // kernels of one captured step
    dbox_profile profile;
    int last_launches = 0;              // kernels launched by the last stepping call (all its steps)
    dbox_event_fn listener = nullptr;
    void* listener_user = nullptr;
    // table contact filters (b2World.SetContactFilter): per world a mode and 64 class rows
    std::vector<int> fmode;
    std::vector<unsigned long long> ftab;
    DBuf<int> d_fmode;
    DBuf<unsigned long long> d_ftab;
    bool filter_dirty = false;
    dbox_world* start_src = nullptr;         // warm-start mode 3: the handle whose contacts give the start
    dbox_presolve_fn presolve = nullptr;     // PreSolve window between Collide and Solve
    void* presolve_user = nullptr;
    std::vector<dbox_presolve_contact> h_presolve;
    cudaEvent_t ev[4];
    bool events_made = false;
    // timed multi-step graph (per-phase events inside the graph)
    cudaGraphExec_t tgraph = nullptr;
    std::vector<cudaEvent_t> tev;
    int t_steps = -1;
    float t_dt = -1.0f;
    int t_vi = -1, t_pi = -1, t_flags = -1;
    int t_launches = 0;                 // kernels of the timed graph
    // world queries: the device index of the broad-phase's fat AABBs
    unsigned long long gen = 0;         // bumped before any device work that may move proxies
    unsigned long long q_gen = ~0ull;   // gen the index was built at
    DBuf<float4> q_box, q_bucket, q_group;
    DBuf<int> q_idx, q_live, q_sidx0, q_sidx1;
    DBuf<unsigned> q_key0, q_key1, q_bitmap;
    int q_bm_words = 0, q_blocks = 0;
    DBuf<unsigned char> q_in, q_out;    // staging of the host-buffer query calls
};

namespace {

void free_device(dbox_world* w) {
    w->d_wi.free(); w->d_wd.free(); w->d_bs.free(); w->d_bst.free(); w->d_body_fix.free();
    w->d_jadj_joint.free(); w->d_jadj_other.free(); w->d_fx.free(); w->d_px.free(); w->d_jt.free();
    w->d_ct.free(); w->d_cworld.free(); w->d_hash.free(); w->d_pairs.free();
    DBuf<int>* ints[] = {&w->s_woken, &w->s_adj_start, &w->s_cursor, &w->s_stack, &w->s_isl_body, &w->s_body_island,
                         &w->s_last, &w->s_isl_bstart, &w->s_isl_cstart, &w->s_isl_jstart, &w->s_isl_flags,
                         &w->s_pcount, &w->s_moved, &w->s_cstate, &w->s_isl_contact, &w->s_level, &w->s_lcur, &w->s_tcand,
                         &w->s_sched_v, &w->s_lvl_v, &w->s_sched_p, &w->s_lvl_p, &w->s_tmp, &w->s_isl_joint,
                         &w->s_accept, &w->g_status};
    for (auto* b : ints) b->free();
    w->s_isl_minsep.free(); w->s_isl_sleep.free();
    w->d_vr.free(); w->d_tvr.free(); w->d_pr.free(); w->d_tpr.free(); w->d_snap.free(); w->d_io.free();
    w->s_vpos.free(); w->d_solve_world.free(); w->d_solve_smem.free();
    w->q_box.free(); w->q_bucket.free(); w->q_group.free(); w->q_idx.free(); w->q_live.free(); w->q_sidx0.free();
    w->q_sidx1.free(); w->q_key0.free(); w->q_key1.free(); w->q_bitmap.free(); w->q_in.free(); w->q_out.free();
    w->q_bm_words = 0;
    w->q_blocks = 0;
    w->q_gen = ~0ull;
    w->d_solve_order.free(); w->d_solve_queue.free();
    w->s_feat.free(); w->s_vsave.free(); w->s_slog.free(); w->s_pend.free();
    w->d_events.free(); w->s_cevt.free();
    w->d_fmode.free(); w->d_ftab.free();
    w->filter_dirty = true;
    w->s_sapk0.free(); w->s_sapk1.free(); w->s_sapi0.free(); w->s_sapi1.free(); w->s_sapbox.free(); w->d_porder.free(); w->s_sapcell.free(); w->d_big.free(); w->n_big = 0;
    w->s_cbody.free(); w->s_adj_items.free(); w->s_isl_pair.free(); w->s_cq.free(); w->s_cvis.free(); w->s_bfl.free(); w->s_sbody.free(); w->d_prof.free();
    if (w->graph) { cudaGraphExecDestroy(w->graph); w->graph = nullptr; }
    if (w->tgraph) { cudaGraphExecDestroy(w->tgraph); w->tgraph = nullptr; }
}

int next_pow2(int v) { int p = 1; while (p < v) p <<= 1; return p; }

// scratch of the learned warm start (features and pending lists per contact slot, sample
// slots per velocity row) and of the measure mode (saved velocities per body), only while
// those modes are on
int alloc_mode_scratch(dbox_world* w) {
    if (w->wi.empty()) return DBOX_OK;
    size_t nc = (size_t)w->total_contacts, nb = (size_t)w->total_bodies, nkx = 0;
    for (const auto& wi : w->wi) nkx = std::max(nkx, (size_t)wi.kx_start + wi.contact_cap + wi.joint_count + 2);
    bool ok = true;
    if (w->ws_mode) {
        if (!w->s_slog.p) ok &= w->s_slog.alloc(nkx) == 0;
        if (!w->s_feat.p) ok &= w->s_feat.alloc((size_t)dg::kFeat * nc) == 0;
        if (!w->s_pend.p) ok &= w->s_pend.alloc(nc) == 0;
    }
    if (w->measure && !w->s_vsave.p) ok &= w->s_vsave.alloc(3 * nb) == 0;
    if (w->listener || w->presolve) {
        if (!w->s_cevt.p) ok &= w->s_cevt.alloc(nc) == 0;
        if (!w->d_events.p) ok &= w->d_events.alloc(4 * nc + 64 * w->wi.size()) == 0;
    }
    if (!ok) return fail(DBOX_ERR_CUDA, "device allocation failed (warm-start / measure scratch)");
    return DBOX_OK;
}

// World-queue mapping: one resident wave of four-warp blocks (as many as fit on every SM);
// each warp owns a fixed region of shared memory (row staging + solver body rows for up to
// solve_cap bodies) and takes worlds from the queue, costliest first (measured costs when
// the autotuner has them, else body counts).
int pack_solve_queue(dbox_world* w) {
    const int W = (int)w->wi.size();
    if (w->nsm <= 0) {
        int dev = 0;
        CU(cudaGetDevice(&dev));
        CU(cudaDeviceGetAttribute(&w->nsm, cudaDevAttrMultiProcessorCount, dev));
    }
    int max_nb = 1;
    for (const auto& wi : w->wi) max_nb = std::max(max_nb, wi.body_count);
    // two blocks per SM: 113 KB of shared memory per block, 4 KB of it static
    const int per_warp_bytes = (113 * 1024 - 4096) / dg::kSolveWarps;
    const int cap_max = (per_warp_bytes - (int)sizeof(float) * dg::kWarpSmemFloats) / 32;
    w->solve_cap = std::min(max_nb, cap_max);
    w->solve_wpb = dg::kSolveWarps;
    w->solve_smem_floats = dg::kSolveWarps * (dg::kWarpSmemFloats + 8 * w->solve_cap);
    int occ = 1 << 30;
    for (const void* k : {dbox_solve_kernel(), dbox_step_fused_kernel()}) {   // the queue's wave fits both
        CU(cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)(sizeof(float) * w->solve_smem_floats)));
        int o = 0;
        CU(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&o, k, dg::kSolveWarps * 32, sizeof(float) * w->solve_smem_floats));
        occ = std::min(occ, o);
    }
    if (occ < 1) return fail(DBOX_ERR_CUDA, "solve kernel does not fit on an SM");
    if (w->solve_bps > 0) occ = std::min(occ, w->solve_bps);
    w->solve_blocks = std::max(1, std::min(w->nsm * occ, (W + dg::kSolveWarps - 1) / dg::kSolveWarps));
    std::vector<int> order(W);
    for (int i = 0; i < W; ++i) order[i] = i;
    const bool measured = (int)w->world_cost.size() == W;
    std::stable_sort(order.begin(), order.end(), [&](int a, int b) {
        if (measured) return w->world_cost[a] > w->world_cost[b];
        return w->wi[a].body_count > w->wi[b].body_count;
    });
    if (w->d_solve_order.alloc(std::max(W, 1)) || w->d_solve_queue.alloc(2 + 4 * (size_t)w->nsm))
        return fail(DBOX_ERR_CUDA, "device allocation failed (solve queue)");
    if (W) CU(cudaMemcpy(w->d_solve_order.p, order.data(), sizeof(int) * W, cudaMemcpyHostToDevice));
    CU(cudaMemset(w->d_solve_queue.p, 0, sizeof(int) * (2 + 4 * (size_t)w->nsm)));
    return DBOX_OK;
}

// Warp slots of the solve kernel (four per block).  Each world's solver body rows and
// island words (32 bytes a body) go to shared memory when they fit the block's budget; worlds are
// placed largest first (first fit over the open blocks), so the biggest worlds sit in
// the lowest blocks and start first, and small worlds fill the remaining room.
int pack_solve_slots(dbox_world* w) {
    if (w->solve_queue_mode) return pack_solve_queue(w);
    const int W = (int)w->wi.size();
    int max_nb = 0;
    for (const auto& wi : w->wi) max_nb = std::max(max_nb, wi.body_count);
    // budget in bodies per block: room for the largest world, at least 1024, and at most
    // 1536 when there are enough worlds to fill the GPU (three blocks per SM stay resident);
    // the front of the block holds each warp's constraint-row staging slots
    const int wpb = w->solve_wpb;
    const int stage_floats = wpb * dg::kWarpSmemFloats;
    const int hard_cap = (227 * 1024 - 1024 - 4096 - 4 * stage_floats) / 32;
    int budget = std::max(1024, max_nb);
    budget = std::min(budget, W >= 3 * 152 ? 1536 : hard_cap);
    if (w->solve_budget > 0) budget = std::min(w->solve_budget, hard_cap);
    std::vector<int> order(W);
    for (int i = 0; i < W; ++i) order[i] = i;
    std::stable_sort(order.begin(), order.end(),
                     [&](int a, int b) { return w->wi[a].body_count > w->wi[b].body_count; });
    std::vector<int> used, count, slot_world, slot_off;
    std::vector<int> open;                  // blocks with a free slot, in creation order
    int placed = 0;
    for (int wid : order) {
        if (placed++ < w->solve_isolate) {   // a block of its own: no other warp competes on that block
            int nbw = w->wi[wid].body_count;
            bool in_smem = nbw <= budget;
            int b = (int)used.size();
            used.push_back(in_smem ? nbw : 0);
            count.push_back(wpb);
            slot_world.resize(used.size() * wpb, -1);
            slot_off.resize(used.size() * wpb, -1);
            slot_world[b * wpb] = wid;
            slot_off[b * wpb] = in_smem ? stage_floats : -1;
            continue;
        }
        int nbw = w->wi[wid].body_count;
        bool in_smem = nbw <= budget;
        int need = in_smem ? nbw : 0;
        int chosen = -1;
        size_t keep = 0;
        for (size_t t = 0; t < open.size(); ++t) {
            int b = open[t];
            if (chosen < 0 && used[b] + need <= budget) chosen = b;
            if (count[b] + (b == chosen) < wpb) open[keep++] = b;   // still has a free slot
        }
        open.resize(keep);
        if (chosen < 0) {
            chosen = (int)used.size();
            used.push_back(0);
            count.push_back(0);
            slot_world.resize(used.size() * wpb, -1);
            slot_off.resize(used.size() * wpb, -1);
            if (wpb > 1) open.push_back(chosen);
        }
        int slot = chosen * wpb + count[chosen]++;
        slot_world[slot] = wid;
        slot_off[slot] = in_smem ? stage_floats + 8 * used[chosen] : -1;
        used[chosen] += need;
    }
    if (used.empty()) {                     // no worlds: one idle block
        used.push_back(0);
        slot_world.assign(wpb, -1);
        slot_off.assign(wpb, -1);
    }
    int max_used = 0;
    for (int u : used) max_used = std::max(max_used, u);
    w->solve_blocks = (int)used.size();
    w->solve_smem_floats = stage_floats + 8 * std::max(max_used, 1);
    if (w->d_solve_world.alloc(slot_world.size()) || w->d_solve_smem.alloc(slot_off.size()))
        return fail(DBOX_ERR_CUDA, "device allocation failed (solve slots)");
    CU(cudaMemcpy(w->d_solve_world.p, slot_world.data(), sizeof(int) * slot_world.size(), cudaMemcpyHostToDevice));
    CU(cudaMemcpy(w->d_solve_smem.p, slot_off.data(), sizeof(int) * slot_off.size(), cudaMemcpyHostToDevice));
    for (const void* k : {dbox_solve_kernel(), dbox_step_fused_kernel()})
        CU(cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)(sizeof(float) * w->solve_smem_floats)));
    return DBOX_OK;
}

// Pull the authoritative dynamic state back to the host mirrors.
int download(dbox_world* w) {
    if (!w->on_device) return 0;
    CU(cudaStreamSynchronize(w->stream));
    int W = (int)w->worlds.size();
    std::vector<dg::WorldDyn> wd(W);
    CU(cudaMemcpy(wd.data(), w->d_wd.p, sizeof(dg::WorldDyn) * W, cudaMemcpyDeviceToHost));
    for (int i = 0; i < W; ++i) {
        HostWorld& hw = w->worlds[i];
        const dg::WorldInfo& wi = w->wi[i];
        hw.wd = wd[i];
        if (!hw.bs.empty())
            CU(cudaMemcpy(hw.bs.data(), w->d_bs.p + wi.body_start, sizeof(dbox_body_state) * hw.bs.size(),
                          cudaMemcpyDeviceToHost));
        if (!hw.px.empty())
            CU(cudaMemcpy(hw.px.data(), w->d_px.p + wi.fix_start, sizeof(dbox_proxy_state) * hw.px.size(),
                          cudaMemcpyDeviceToHost));
        if (!hw.jt.empty())
            CU(cudaMemcpy(hw.jt.data(), w->d_jt.p + wi.joint_start, sizeof(dg::DJoint) * hw.jt.size(),
                          cudaMemcpyDeviceToHost));
        hw.ct.resize(hw.wd.contact_count);
        if (!hw.ct.empty())
            CU(cudaMemcpy(hw.ct.data(), w->d_ct.p + wi.contact_start, sizeof(dbox_contact_state) * hw.ct.size(),
                          cudaMemcpyDeviceToHost));
        // device fixture/joint indices are global; host mirrors keep world-local ones
        for (auto& c : hw.ct) { c.fixture_a -= wi.fix_start; c.fixture_b -= wi.fix_start; }
        for (auto& j : hw.jt) {
            j.body_a -= wi.body_start;
            j.body_b -= wi.body_start;
            if (j.type == dg::kGearJoint) {
                j.body_c -= wi.body_start;
                j.body_d -= wi.body_start;
            }
        }
    }
    w->on_device = false;
    w->mirrors_fresh = true;
    return 0;
}

// Lay out every world in the batch and copy it to the device.
int upload(dbox_world* w) {
    free_device(w);
    int W = (int)w->worlds.size();
    w->wi.assign(W, dg::WorldInfo());
    int nb = 0, nf = 0, nj = 0, nc = 0, nh = 0, np = 0, nbx = 0, nkx = 0;
    int cpb = w->caps.contacts_per_body > 0 ? w->caps.contacts_per_body : 8;
    std::vector<int> porder, big;
    for (int i = 0; i < W; ++i) {
        HostWorld& hw = w->worlds[i];
        dg::WorldInfo& wi = w->wi[i];
        int b = (int)hw.bs.size(), f = (int)hw.fx.size(), j = (int)hw.jt.size();
        int cap = cpb * b + 64;
        if (cap < (int)hw.ct.size() * 2) cap = (int)hw.ct.size() * 2;
        wi.body_start = nb; wi.body_count = b;
        wi.fix_start = nf; wi.fix_count = f;
        wi.joint_start = nj; wi.joint_count = j;
        wi.contact_start = nc; wi.contact_cap = cap;
        wi.hash_start = nh; wi.hash_cap = next_pow2(2 * cap);
        wi.pair_start = np; wi.pair_cap = 16 * f + 64;
        wi.bx_start = nbx;
        wi.kx_start = nkx;
        wi.snap_start = nc;
        // broad-phase walk order: fixtures by proxy id (no-proxy fixtures last); the plain
        // fixture order while the ids rise with the fixture index (always, without destruction)
        wi.pair_block = f >= kPairBlockFixtures ? 1 : 0;
        if (wi.pair_block) big.push_back(i);
        wi.proxy_order = 0;
        for (int i = 0, last = -1; i < f; ++i) {
            const int id = hw.px[i].proxy_id;
            if (id < 0) continue;
            if (id < last) wi.proxy_order = 1;
            last = id;
        }
        porder.resize(nf + f);
        for (int i = 0; i < f; ++i) porder[nf + i] = i;
        if (wi.proxy_order)
            std::stable_sort(porder.begin() + nf, porder.end(), [&](int a, int c) {
                const unsigned ia = (unsigned)hw.px[a].proxy_id, ic = (unsigned)hw.px[c].proxy_id;   // -1 sorts last
                return ia < ic;
            });
        nb += b; nf += f; nj += j; nc += cap; nh += wi.hash_cap; np += wi.pair_cap; nbx += b + 1; nkx += cap + j + 2;
    }
    w->total_bodies = nb; w->total_fixtures = nf; w->total_joints = nj; w->total_contacts = nc;
    // flatten
    std::vector<dg::WorldDyn> wd(W);
    std::vector<dbox_body_state> bs(nb);
    std::vector<dg::BodyStatic> bst(nb);
    std::vector<int> body_fix, jadj_joint, jadj_other;
    std::vector<dg::DFixture> fx(nf);
    std::vector<dbox_proxy_state> px(nf);
    std::vector<dg::DJoint> jt(nj);
    std::vector<dbox_contact_state> ct(nc);
    std::vector<int> cworld(nc);
    memset(ct.data(), 0, sizeof(dbox_contact_state) * ct.size());
    for (int i = 0; i < W; ++i) {
        HostWorld& hw = w->worlds[i];
        const dg::WorldInfo& wi = w->wi[i];
        wd[i] = hw.wd;
        wd[i].contact_count = (int)hw.ct.size();
        wd[i].flags = (hw.wd.flags & ~4u) | (w->autoclear ? 4u : 0u);
        // joint adjacency, newest joint first (b2world.d:226-242 head insertion)
        std::vector<std::vector<std::pair<int, int>>> jadj(hw.bs.size());
        for (int j = 0; j < (int)hw.jt.size(); ++j) {
            if (hw.jt[j].type < 0) continue;                            // destroyed
            jadj[hw.jt[j].body_a].push_back({j, hw.jt[j].body_b});
            jadj[hw.jt[j].body_b].push_back({j, hw.jt[j].body_a});
        }
        for (int b = 0; b < (int)hw.bs.size(); ++b) {
            bs[wi.body_start + b] = hw.bs[b];
            dg::BodyStatic s = hw.bst[b];
            s.world = i;
            s.fix_start = (int)body_fix.size();
            s.fix_count = (int)hw.body_fix[b].size();
            for (int f : hw.body_fix[b]) body_fix.push_back(wi.fix_start + f);
            s.jadj_start = (int)jadj_joint.size();
            s.jadj_count = (int)jadj[b].size();
            for (int e = (int)jadj[b].size() - 1; e >= 0; --e) {
                jadj_joint.push_back(wi.joint_start + jadj[b][e].first);
                jadj_other.push_back(wi.body_start + jadj[b][e].second);
            }
            bst[wi.body_start + b] = s;
        }
        for (int f = 0; f < (int)hw.fx.size(); ++f) {
            dg::DFixture d = hw.fx[f];
            d.body += wi.body_start;
            fx[wi.fix_start + f] = d;
            px[wi.fix_start + f] = hw.px[f];
        }
        for (int j = 0; j < (int)hw.jt.size(); ++j) {
            dg::DJoint d = hw.jt[j];
            d.body_a += wi.body_start;
            d.body_b += wi.body_start;
            if (d.type == dg::kGearJoint) {
                d.body_c += wi.body_start;
                d.body_d += wi.body_start;
            }
            jt[wi.joint_start + j] = d;
        }
        for (int k = 0; k < (int)hw.ct.size(); ++k) {
            dbox_contact_state c = hw.ct[k];
            c.fixture_a += wi.fix_start;
            c.fixture_b += wi.fix_start;
            ct[wi.contact_start + k] = c;
        }
        for (int k = 0; k < wi.contact_cap; ++k) cworld[wi.contact_start + k] = i;
    }
    bool ok = true;
    ok &= w->d_wi.alloc(W) == 0;
    ok &= w->d_wd.alloc(W) == 0;
    ok &= w->d_bs.alloc(nb) == 0;
    ok &= w->d_bst.alloc(nb) == 0;
    ok &= w->d_body_fix.alloc(body_fix.size()) == 0;
    ok &= w->d_jadj_joint.alloc(jadj_joint.size()) == 0;
    ok &= w->d_jadj_other.alloc(jadj_other.size()) == 0;
    ok &= w->d_fx.alloc(nf) == 0;
    ok &= w->d_px.alloc(nf) == 0;
    ok &= w->d_jt.alloc(nj) == 0;
    ok &= w->d_ct.alloc(nc) == 0;
    ok &= w->d_cworld.alloc(nc) == 0;
    ok &= w->d_hash.alloc(nh) == 0;
    ok &= w->d_pairs.alloc(np) == 0;
    ok &= w->s_woken.alloc(nb) == 0;
    ok &= w->s_adj_start.alloc(nbx) == 0;
    ok &= w->s_cursor.alloc(nb) == 0;
    ok &= w->s_stack.alloc(nb) == 0;
    ok &= w->s_isl_body.alloc(nb) == 0;
    ok &= w->s_body_island.alloc(nb) == 0;
    ok &= w->s_last.alloc(nb) == 0;
    ok &= w->s_isl_bstart.alloc(nbx) == 0;
    ok &= w->s_isl_cstart.alloc(nbx) == 0;
    ok &= w->s_isl_jstart.alloc(nbx) == 0;
    ok &= w->s_isl_flags.alloc(nb) == 0;
    ok &= w->s_isl_minsep.alloc(nb) == 0;
    ok &= w->s_isl_sleep.alloc(nb) == 0;
    ok &= w->s_pcount.alloc(nf) == 0;
    ok &= w->s_moved.alloc(nf) == 0;
    ok &= w->s_sapk0.alloc(nf) == 0 && w->s_sapk1.alloc(nf) == 0;
    ok &= w->s_sapi0.alloc(nf) == 0 && w->s_sapi1.alloc(nf) == 0;
    ok &= w->s_sapbox.alloc(nf) == 0;
    ok &= w->d_porder.alloc(nf) == 0;
    ok &= w->s_sapcell.alloc(8 * (size_t)nf + 130 * (size_t)W) == 0;
    ok &= w->d_big.alloc(big.size()) == 0;
    w->n_big = (int)big.size();
    ok &= w->s_cstate.alloc(nc) == 0;
    ok &= w->s_adj_items.alloc(2 * (size_t)nc) == 0;
    ok &= w->s_isl_pair.alloc(nc) == 0;
    ok &= w->s_lcur.alloc(nkx) == 0;
    ok &= w->s_tcand.alloc(nc) == 0;
    ok &= w->s_isl_contact.alloc(nc) == 0;
    ok &= w->s_level.alloc(nkx) == 0;
    ok &= w->s_sched_v.alloc(nkx) == 0;
    ok &= w->s_lvl_v.alloc(nkx) == 0;
    ok &= w->s_sched_p.alloc(nkx) == 0;
    ok &= w->s_lvl_p.alloc(nkx) == 0;
    ok &= w->s_tmp.alloc(nkx) == 0;
    ok &= w->s_isl_joint.alloc(nj) == 0;
    ok &= w->s_accept.alloc(np) == 0;
    ok &= w->g_status.alloc(1) == 0;
    ok &= w->d_vr.alloc(nkx) == 0;
    ok &= w->d_pr.alloc(nkx) == 0;
    ok &= w->d_tvr.alloc((size_t)dg::kMaxTOIContacts * W) == 0;
    ok &= w->d_tpr.alloc((size_t)dg::kMaxTOIContacts * W) == 0;
    ok &= w->s_vpos.alloc(nc) == 0;
    ok &= w->d_snap.alloc(nc) == 0;
    ok &= w->d_io.alloc(3 * (size_t)nb) == 0;
    ok &= w->s_cbody.alloc(nc) == 0;
    ok &= w->s_cq.alloc(nc) == 0;
    ok &= w->s_cvis.alloc(nc) == 0;
    ok &= w->s_bfl.alloc(nb) == 0;
    ok &= w->s_sbody.alloc(6 * (size_t)nb) == 0;
    ok &= w->d_prof.alloc((size_t)dg::kProfSlots * W) == 0;
    if (!ok) { free_device(w); return fail(DBOX_ERR_CUDA, "device allocation failed (%d bodies, %d contact slots)", nb, nc); }
    if (pack_solve_slots(w) != DBOX_OK) { free_device(w); return DBOX_ERR_CUDA; }
    if (alloc_mode_scratch(w) != DBOX_OK) { free_device(w); return DBOX_ERR_CUDA; }
    CU(cudaMemcpy(w->d_wi.p, w->wi.data(), sizeof(dg::WorldInfo) * W, cudaMemcpyHostToDevice));
    CU(cudaMemcpy(w->d_wd.p, wd.data(), sizeof(dg::WorldDyn) * W, cudaMemcpyHostToDevice));
    if (nb) {
        CU(cudaMemcpy(w->d_bs.p, bs.data(), sizeof(dbox_body_state) * nb, cudaMemcpyHostToDevice));
        CU(cudaMemcpy(w->d_bst.p, bst.data(), sizeof(dg::BodyStatic) * nb, cudaMemcpyHostToDevice));
    }
    if (!body_fix.empty()) CU(cudaMemcpy(w->d_body_fix.p, body_fix.data(), sizeof(int) * body_fix.size(), cudaMemcpyHostToDevice));
    if (!jadj_joint.empty()) {
        CU(cudaMemcpy(w->d_jadj_joint.p, jadj_joint.data(), sizeof(int) * jadj_joint.size(), cudaMemcpyHostToDevice));
        CU(cudaMemcpy(w->d_jadj_other.p, jadj_other.data(), sizeof(int) * jadj_other.size(), cudaMemcpyHostToDevice));
    }
    if (nf) {
        CU(cudaMemcpy(w->d_fx.p, fx.data(), sizeof(dg::DFixture) * nf, cudaMemcpyHostToDevice));
        CU(cudaMemcpy(w->d_px.p, px.data(), sizeof(dbox_proxy_state) * nf, cudaMemcpyHostToDevice));
        CU(cudaMemcpy(w->d_porder.p, porder.data(), sizeof(int) * nf, cudaMemcpyHostToDevice));
        if (!big.empty()) CU(cudaMemcpy(w->d_big.p, big.data(), sizeof(int) * big.size(), cudaMemcpyHostToDevice));
    }
    if (nj) CU(cudaMemcpy(w->d_jt.p, jt.data(), sizeof(dg::DJoint) * nj, cudaMemcpyHostToDevice));
    if (nc) {
        CU(cudaMemcpy(w->d_ct.p, ct.data(), sizeof(dbox_contact_state) * nc, cudaMemcpyHostToDevice));
        CU(cudaMemcpy(w->d_cworld.p, cworld.data(), sizeof(int) * nc, cudaMemcpyHostToDevice));
    }
    CU(cudaMemset(w->g_status.p, 0, sizeof(int)));
    w->on_device = true;
    w->dirty = false;
    return 0;
}

// the table contact filters on the device (nothing while every world keeps the default rule)
int sync_filter(dbox_world* w) {
    if (!w->filter_dirty) return 0;
    bool any = false;
    for (int m : w->fmode) any |= m != 0;
    if (!any) {
        w->d_fmode.free();
        w->d_ftab.free();
    } else {
        if (!w->d_fmode.p && w->d_fmode.alloc(w->fmode.size())) return fail(DBOX_ERR_CUDA, "filter allocation failed");
        if (!w->d_ftab.p && w->d_ftab.alloc(w->ftab.size())) return fail(DBOX_ERR_CUDA, "filter allocation failed");
        CU(cudaMemcpy(w->d_fmode.p, w->fmode.data(), sizeof(int) * w->fmode.size(), cudaMemcpyHostToDevice));
        CU(cudaMemcpy(w->d_ftab.p, w->ftab.data(), sizeof(unsigned long long) * w->ftab.size(), cudaMemcpyHostToDevice));
    }
    w->filter_dirty = false;
    return 0;
}

int ensure_device(dbox_world* w) {
    w->mirrors_fresh = false;              // device work follows
    ++w->gen;                              // and may move proxies: the query index goes stale
    if (w->dirty || !w->on_device) {
        int rc = download(w);
        if (rc) return rc;
        rc = upload(w);
        if (rc) return rc;
        if (w->n_big > 0) CU((cudaError_t)dbox_big_solve_init(&w->big_cluster));
    }
    return sync_filter(w);
}

dg::Ctx make_ctx(dbox_world* w, float dt, int vi, int pi) {
    dg::Ctx x;
    memset(&x, 0, sizeof(x));
    x.W = (int)w->worlds.size();
    x.total_bodies = w->total_bodies;
    x.total_fixtures = w->total_fixtures;
    x.total_contacts = w->total_contacts;
    x.total_joints = w->total_joints;
    x.wi = w->d_wi.p;
    x.wd = w->d_wd.p;
    x.bs = w->d_bs.p;
    x.bst = w->d_bst.p;
    x.body_fix = w->d_body_fix.p;
    x.jadj_joint = w->d_jadj_joint.p;
    x.jadj_other = w->d_jadj_other.p;
    x.fx = w->d_fx.p;
    x.px = w->d_px.p;
    x.jt = w->d_jt.p;
    x.ct = w->d_ct.p;
    x.c_world = w->d_cworld.p;
    x.hash = w->d_hash.p;
    x.pairs = w->d_pairs.p;
    x.s_woken = w->s_woken.p;
    x.s_adj_start = w->s_adj_start.p;
    x.s_cursor = w->s_cursor.p;
    x.s_stack = w->s_stack.p;
    x.s_isl_body = w->s_isl_body.p;
    x.s_body_island = w->s_body_island.p;
    x.s_last = w->s_last.p;
    x.s_isl_bstart = w->s_isl_bstart.p;
    x.s_isl_cstart = w->s_isl_cstart.p;
    x.s_isl_jstart = w->s_isl_jstart.p;
    x.s_isl_minsep = w->s_isl_minsep.p;
    x.s_isl_flags = w->s_isl_flags.p;
    x.s_isl_sleep = w->s_isl_sleep.p;
    x.s_pcount = w->s_pcount.p;
    x.s_moved = w->s_moved.p;
    x.s_cstate = w->s_cstate.p;
    x.s_adj_items = w->s_adj_items.p;
    x.s_isl_pair = w->s_isl_pair.p;
    x.s_lcur = w->s_lcur.p;
    x.s_tcand = w->s_tcand.p;
    x.s_isl_contact = w->s_isl_contact.p;
    x.s_level = w->s_level.p;
    x.s_sched_v = w->s_sched_v.p;
    x.s_lvl_v = w->s_lvl_v.p;
    x.s_sched_p = w->s_sched_p.p;
    x.s_lvl_p = w->s_lvl_p.p;
    x.s_tmp = w->s_tmp.p;
    x.s_isl_joint = w->s_isl_joint.p;
    x.s_accept = w->s_accept.p;
    x.vr = w->d_vr.p;
    x.pr = w->d_pr.p;
    x.tvr = w->d_tvr.p;
    x.tpr = w->d_tpr.p;
    x.s_vpos = w->s_vpos.p;
    x.solve_world = w->d_solve_world.p;
    x.solve_smem = w->d_solve_smem.p;
    x.solve_blocks = w->solve_blocks;
    x.solve_wpb = w->solve_wpb;
    x.solve_smem_floats = w->solve_smem_floats;
    x.solve_order = w->d_solve_order.p;
    x.solve_queue = w->solve_queue_mode ? w->d_solve_queue.p : nullptr;
    x.solve_heavy = std::min(w->solve_heavy, (int)w->worlds.size());
    x.solve_exclusive = w->solve_exclusive;
    x.solve_cap = w->solve_cap;
    x.solve_nsm = w->nsm;
    x.snap = w->d_snap.p;
    x.s_cbody = w->s_cbody.p;
    x.s_cq = w->s_cq.p;
    x.s_cvis = w->s_cvis.p;
    x.s_bfl = w->s_bfl.p;
    x.s_sbody = w->s_sbody.p;
    x.dt = dt;
    x.inv_dt = dt > 0.0f ? 1.0f / dt : 0.0f;                            // b2world.d:383-390
    x.vel_iters = vi;
    x.pos_iters = pi;
    x.gravity = w->gravity;
    x.warm_starting = w->warm;
    x.continuous = w->continuous;
    x.sub_stepping = w->substep;
    x.allow_sleep = w->allow_sleep;
    x.record_events = (w->listener || w->presolve) ? 1 : 0;
    x.g_status = w->g_status.p;
    x.prof = w->profiling ? w->d_prof.p : nullptr;
    x.ws_mode = w->ws_mode;
    if (w->ws_mode == 2 && w->mlp) dbox_mlp_device_view(w->mlp, &x.mlp);
    x.samples = w->d_samples.p;
    x.start_ct = (w->ws_mode == 3 && w->start_src) ? w->start_src->d_ct.p : nullptr;
    x.sample_count = w->d_sample_count.p;
    x.sample_cap = w->sample_cap;
    x.s_slog = w->s_slog.p;
    x.s_feat = w->s_feat.p;
    x.s_pend = w->s_pend.p;
    x.measure = w->measure;
    x.wait_polls = w->wait_polls;
    x.fmode = w->d_fmode.p;
    x.ftab = w->d_ftab.p;
    x.s_vsave = w->s_vsave.p;
    x.events = w->d_events.p;
    x.s_sapk[0] = w->s_sapk0.p;
    x.s_sapk[1] = w->s_sapk1.p;
    x.s_sapi[0] = w->s_sapi0.p;
    x.s_sapi[1] = w->s_sapi1.p;
    x.s_sapbox = w->s_sapbox.p;
    x.proxy_order = w->d_porder.p;
    x.s_sapcell = w->s_sapcell.p;
    x.big_worlds = w->d_big.p;
    x.n_big = w->n_big;
    x.big_block = (w->n_big > 0 && w->island_solver == 0) ? 1 : 0;
    x.big_cluster = w->big_cluster;
    x.s_cevt = w->s_cevt.p;
    return x;
}

int check_status(dbox_world* w) {
    int st = 0;
    CU(cudaMemcpyAsync(&st, w->g_status.p, sizeof(int), cudaMemcpyDeviceToHost, w->stream));
    CU(cudaStreamSynchronize(w->stream));
    if (st) {
        CU(cudaMemsetAsync(w->g_status.p, 0, sizeof(int), w->stream));
        for (int code = 1; code < 31; ++code)
            if (st & (1 << code)) return fail(-code, "device step reported status %d (bits 0x%x)", -code, st);
    }
    return 0;
}

void fill_body_state(const dbox_body_def* d, dbox_body_state* s, dg::BodyStatic* st) {
    memset(s, 0, sizeof(*s));                                           // b2body.d:1030-1115
    uint32_t f = 0;
    if (d->bullet) f |= dg::kBodyBullet;
    if (d->fixed_rotation) f |= dg::kBodyFixedRotation;
    if (d->allow_sleep) f |= dg::kBodyAutoSleep;
    if (d->awake) f |= dg::kBodyAwake;
    if (d->active) f |= dg::kBodyActive;
    s->flags = f;
    s->type = d->type;
    hg::Rot q = hg::rot(d->angle);
    s->xf[0] = d->position.x; s->xf[1] = d->position.y; s->xf[2] = q.s; s->xf[3] = q.c;
    s->sweep[0] = 0.0f; s->sweep[1] = 0.0f;
    s->sweep[2] = d->position.x; s->sweep[3] = d->position.y;
    s->sweep[4] = d->position.x; s->sweep[5] = d->position.y;
    s->sweep[6] = d->angle; s->sweep[7] = d->angle; s->sweep[8] = 0.0f;
    s->vel[0] = d->linear_velocity.x; s->vel[1] = d->linear_velocity.y; s->vel[2] = d->angular_velocity;
    if (d->type == DBOX_DYNAMIC_BODY) { s->mass[0] = 1.0f; s->mass[1] = 1.0f; }
    memset(st, 0, sizeof(*st));
    st->lin_damping = d->linear_damping;
    st->ang_damping = d->angular_damping;
    st->gravity_scale = d->gravity_scale;
}

// b2Body.ResetMassData (b2body.d:555-625)
bool body_gone(const HostWorld& hw, int b) { return b < (int)hw.body_dead.size() && hw.body_dead[b]; }

void reset_mass(HostWorld& hw, int b) {
    dbox_body_state& s = hw.bs[b];
    float mass = 0.0f, invMass = 0.0f, I = 0.0f, invI = 0.0f;
    s.sweep[0] = 0.0f; s.sweep[1] = 0.0f;
    if (s.type == DBOX_STATIC_BODY || s.type == DBOX_KINEMATIC_BODY) {
        s.sweep[2] = s.xf[0]; s.sweep[3] = s.xf[1];
        s.sweep[4] = s.xf[0]; s.sweep[5] = s.xf[1];
        s.sweep[6] = s.sweep[7];
        s.mass[0] = s.mass[1] = s.mass[2] = s.mass[3] = 0.0f;
        return;
    }
    hg::V2 lc = hg::mk(0.0f, 0.0f);
    for (int f : hw.body_fix[b]) {
        const dg::DFixture& fx = hw.fx[f];
        if (fx.density == 0.0f) continue;
        hg::Mass md;
        if (fx.type == dg::kShapeCircle) md = hg::circle_mass(hg::mk(fx.v[0].x, fx.v[0].y), fx.radius, fx.density);
        else if (fx.type == dg::kShapeEdge) {                           // b2EdgeShape.ComputeMass: no mass
            md.mass = 0.0f;
            md.center = hg::scl(0.5f, hg::add(hg::mk(fx.v[0].x, fx.v[0].y), hg::mk(fx.v[1].x, fx.v[1].y)));
            md.I = 0.0f;
        } else {
            hg::Poly p;
            p.count = fx.count;
            for (int i = 0; i < fx.count; ++i) { p.v[i] = hg::mk(fx.v[i].x, fx.v[i].y); }
            md = hg::poly_mass(p, fx.density);
        }
        mass += md.mass;
        lc = hg::add(lc, hg::scl(md.mass, md.center));
        I += md.I;
    }
    if (mass > 0.0f) {
        invMass = 1.0f / mass;
        lc.x *= invMass;
        lc.y *= invMass;
    } else {
        mass = 1.0f;
        invMass = 1.0f;
    }
    if (I > 0.0f && (s.flags & dg::kBodyFixedRotation) == 0) {
        I -= mass * hg::dot(lc, lc);
        invI = 1.0f / I;
    } else {
        I = 0.0f;
        invI = 0.0f;
    }
    hg::V2 oldCenter = hg::mk(s.sweep[4], s.sweep[5]);
    s.sweep[0] = lc.x; s.sweep[1] = lc.y;
    hg::Rot q; q.s = s.xf[2]; q.c = s.xf[3];
    hg::V2 c = hg::xmul(hg::mk(s.xf[0], s.xf[1]), q, lc);
    s.sweep[2] = s.sweep[4] = c.x;
    s.sweep[3] = s.sweep[5] = c.y;
    hg::V2 d = hg::sub(c, oldCenter);
    float wv = s.vel[2];
    s.vel[0] += -wv * d.y;                                             // b2Cross(w, c - oldCenter)
    s.vel[1] += wv * d.x;
    s.mass[0] = mass; s.mass[1] = invMass; s.mass[2] = I; s.mass[3] = invI;
}

bool build_fixture(const dbox_shape_def* sd, dg::DFixture* f) {
    memset(f, 0, sizeof(*f));
    switch (sd->kind) {
    case DBOX_SHAPE_CIRCLE:
        f->type = dg::kShapeCircle;
        f->count = 1;
        f->radius = sd->radius;
        f->v[0] = make_float2(sd->center.x, sd->center.y);
        return true;
    case DBOX_SHAPE_POLYGON:
    case DBOX_SHAPE_BOX:
    case DBOX_SHAPE_ORIENTED_BOX: {
        hg::Poly p;
        if (sd->kind == DBOX_SHAPE_POLYGON) {
            hg::V2 in[8];
            if (sd->count < 3 || sd->count > 8) return false;
            for (int i = 0; i < sd->count; ++i) in[i] = hg::mk(sd->vertices[i].x, sd->vertices[i].y);
            if (!hg::set_hull(p, in, sd->count)) return false;
        } else if (sd->kind == DBOX_SHAPE_BOX) {
            hg::set_as_box(p, sd->hx, sd->hy);
        } else {
            hg::set_as_box(p, sd->hx, sd->hy, hg::mk(sd->center.x, sd->center.y), sd->angle);
        }
        f->type = dg::kShapePolygon;
        f->count = p.count;
        f->radius = 2.0f * 0.005f;                                      // b2_polygonRadius
        for (int i = 0; i < p.count; ++i) {
            f->v[i] = make_float2(p.v[i].x, p.v[i].y);
            f->n[i] = make_float2(p.n[i].x, p.n[i].y);
        }
        f->centroid = make_float2(p.centroid.x, p.centroid.y);
        return true;
    }
    case DBOX_SHAPE_EDGE:                                               // b2EdgeShape.Set + ghost vertices (b2edgeshape.d)
        f->type = dg::kShapeEdge;
        f->count = 2;
        f->radius = 2.0f * 0.005f;                                      // b2_polygonRadius
        f->v[0] = make_float2(sd->vertices[0].x, sd->vertices[0].y);
        f->v[1] = make_float2(sd->vertices[1].x, sd->vertices[1].y);
        f->edge_flags = sd->count & 3;
        f->v[2] = (sd->count & 1) ? make_float2(sd->vertices[2].x, sd->vertices[2].y) : make_float2(0.0f, 0.0f);
        f->v[3] = (sd->count & 2) ? make_float2(sd->vertices[3].x, sd->vertices[3].y) : make_float2(0.0f, 0.0f);
        return true;
    default:
        return false;
    }
}

// polygon / circle AABB at a transform (b2polygonshape.d:356-373, b2circleshape.d:110-117)
void host_aabb(const dg::DFixture& f, const dbox_body_state& b, float out[4]) {
    hg::Rot q; q.s = b.xf[2]; q.c = b.xf[3];
    hg::V2 p = hg::mk(b.xf[0], b.xf[1]);
    if (f.type == dg::kShapeCircle) {
        hg::V2 c = hg::add(p, hg::rmul(q, hg::mk(f.v[0].x, f.v[0].y)));
        out[0] = c.x - f.radius; out[1] = c.y - f.radius; out[2] = c.x + f.radius; out[3] = c.y + f.radius;
        return;
    }
    hg::V2 lo = hg::xmul(p, q, hg::mk(f.v[0].x, f.v[0].y)), hi = lo;
    for (int i = 1; i < f.count; ++i) {
        hg::V2 v = hg::xmul(p, q, hg::mk(f.v[i].x, f.v[i].y));
        lo.x = lo.x < v.x ? lo.x : v.x; lo.y = lo.y < v.y ? lo.y : v.y;
        hi.x = hi.x > v.x ? hi.x : v.x; hi.y = hi.y > v.y ? hi.y : v.y;
    }
    out[0] = lo.x - f.radius; out[1] = lo.y - f.radius; out[2] = hi.x + f.radius; out[3] = hi.y + f.radius;
}

int create_fixture(HostWorld& hw, int body, const dbox_shape_def* shape, const dbox_fixture_def* def) {
    dg::DFixture f;
    if (!build_fixture(shape, &f)) return -1;
    f.body = body;
    f.friction = def->friction;
    f.restitution = def->restitution;
    f.density = def->density;
    f.sensor = def->is_sensor ? 1 : 0;
    f.filter = (uint32_t)def->category_bits | ((uint32_t)def->mask_bits << 16);
    f.group = def->group_index;
    int idx = (int)hw.fx.size();
    hw.fx.push_back(f);
    dbox_proxy_state p;
    memset(&p, 0, sizeof(p));
    p.proxy_id = -1;
    if (hw.bs[body].flags & dg::kBodyActive) {                          // b2fixture.d:450-465 + b2dynamictree.d:110-124
        float a[4];
        host_aabb(f, hw.bs[body], a);
        p.fat_aabb[0] = a[0] - 0.1f; p.fat_aabb[1] = a[1] - 0.1f;
        p.fat_aabb[2] = a[2] + 0.1f; p.fat_aabb[3] = a[3] + 0.1f;
        p.moved = 1;
        p.proxy_id = hw.ids.create();
    }
    hw.px.push_back(p);
    hw.body_fix[body].insert(hw.body_fix[body].begin(), idx);
    if (f.density > 0.0f) reset_mass(hw, body);
    hw.wd.flags |= 1u;                                                  // e_newFixture
    return idx;
}

// append a joint (joint lists are rebuilt newest first from creation order at upload) and
// flag the contacts between its bodies when they may not collide (b2world.d:246-258)
int link_joint(HostWorld& hw, const dg::DJoint& j) {
    int idx = (int)hw.jt.size();
    hw.jt.push_back(j);
    if (!j.collide_connected) {
        for (auto& c : hw.ct) {
            int A = hw.fx[c.fixture_a].body, B = hw.fx[c.fixture_b].body;
            if ((A == j.body_a && B == j.body_b) || (A == j.body_b && B == j.body_a)) c.flags |= dg::kContactFilter;
        }
    }
    return idx;
}

int create_joint(HostWorld& hw, const dbox_revolute_def* d) {
    int nb = (int)hw.bs.size();
    if (d->body_a < 0 || d->body_a >= nb || d->body_b < 0 || d->body_b >= nb || d->body_a == d->body_b ||
        body_gone(hw, d->body_a) || body_gone(hw, d->body_b)) return -1;
    dg::DJoint j;
    memset(&j, 0, sizeof(j));
    j.body_a = d->body_a;
    j.body_b = d->body_b;
    j.collide_connected = d->collide_connected ? 1 : 0;
    j.local_anchor_a = make_float2(d->local_anchor_a.x, d->local_anchor_a.y);
    j.local_anchor_b = make_float2(d->local_anchor_b.x, d->local_anchor_b.y);
    j.reference_angle = d->reference_angle;
    j.enable_limit = d->enable_limit ? 1 : 0;
    j.lower_angle = d->lower_angle;
    j.upper_angle = d->upper_angle;
    j.enable_motor = d->enable_motor ? 1 : 0;
    j.motor_speed = d->motor_speed;
    j.max_motor_torque = d->max_motor_torque;
    j.type = dg::kRevoluteJoint;
    return link_joint(hw, j);
}

// b2World.CreateJoint with a b2DistanceJointDef (b2world.d:196-261, b2distancejoint.d:122-133)
int create_distance_joint(HostWorld& hw, const dbox_distance_def* d) {
    int nb = (int)hw.bs.size();
    if (d->body_a < 0 || d->body_a >= nb || d->body_b < 0 || d->body_b >= nb || d->body_a == d->body_b ||
        body_gone(hw, d->body_a) || body_gone(hw, d->body_b)) return -1;
    dg::DJoint j;
    memset(&j, 0, sizeof(j));
    j.type = dg::kDistanceJoint;
    j.body_a = d->body_a;
    j.body_b = d->body_b;
    j.collide_connected = d->collide_connected ? 1 : 0;
    j.local_anchor_a = make_float2(d->local_anchor_a.x, d->local_anchor_a.y);
    j.local_anchor_b = make_float2(d->local_anchor_b.x, d->local_anchor_b.y);
    j.length = d->length;
    j.frequency_hz = d->frequency_hz;
    j.damping_ratio = d->damping_ratio;
    return link_joint(hw, j);
}

int prepare_edit(dbox_world* w) {
    if (w->on_device) {
        int rc = download(w);
        if (rc) return rc;
    }
    w->dirty = true;
    if (w->graph) { cudaGraphExecDestroy(w->graph); w->graph = nullptr; }
    if (w->tgraph) { cudaGraphExecDestroy(w->tgraph); w->tgraph = nullptr; }
    return 0;
}

}  // namespace

extern "C" {

const char* dbox_last_error(void) { return g_last_error.c_str(); }

void dbox_body_def_default(dbox_body_def* d) {
    memset(d, 0, sizeof(*d));
    d->type = DBOX_STATIC_BODY;
    d->allow_sleep = 1;
    d->awake = 1;
    d->active = 1;
    d->gravity_scale = 1.0f;
}

void dbox_fixture_def_default(dbox_fixture_def* d) {
    memset(d, 0, sizeof(*d));
    d->friction = 0.2f;
    d->category_bits = 0x0001;
    d->mask_bits = 0xFFFF;
}

int32_t dbox_world_create(dbox_vec2 gravity, int32_t n_worlds, const dbox_world_caps* caps, dbox_world** out) {
    if (!out || n_worlds < 1) return fail(DBOX_ERR_INVALID, "dbox_world_create: bad arguments");
    dbox_world* w = new dbox_world();
    w->gravity = make_float2(gravity.x, gravity.y);
    w->worlds.resize(n_worlds);
    memset(&w->caps, 0, sizeof(w->caps));
    if (caps) w->caps = *caps;
    memset(&w->profile, 0, sizeof(w->profile));
    if (cudaStreamCreateWithFlags(&w->stream, cudaStreamNonBlocking) != cudaSuccess) {
        delete w;
        return fail(DBOX_ERR_CUDA, "cudaStreamCreate failed (is a GPU visible?)");
    }
    *out = w;
    return DBOX_OK;
}

int32_t dbox_world_destroy(dbox_world* w) {
    if (!w) return DBOX_ERR_INVALID;
    free_device(w);
    for (auto& e : w->tev) cudaEventDestroy(e);
    if (w->events_made) for (auto& e : w->ev) cudaEventDestroy(e);
    if (w->stream) cudaStreamDestroy(w->stream);
    delete w;
    return DBOX_OK;
}

int32_t dbox_body_create(dbox_world* w, int32_t world, const dbox_body_def* def, int32_t* out_body) {
    if (!w || !def || world < 0 || world >= (int)w->worlds.size()) return fail(DBOX_ERR_INVALID, "dbox_body_create: bad arguments");
    int rc = prepare_edit(w);
    if (rc) return rc;
    HostWorld& hw = w->worlds[world];
    dbox_body_state s;
    dg::BodyStatic st;
    fill_body_state(def, &s, &st);
    hw.bs.push_back(s);
    hw.bst.push_back(st);
    hw.body_fix.emplace_back();
    if (out_body) *out_body = (int)hw.bs.size() - 1;
    return DBOX_OK;
}

int32_t dbox_fixture_create(dbox_world* w, int32_t world, int32_t body, const dbox_shape_def* shape,
                            const dbox_fixture_def* def, int32_t* out_fixture) {
    if (!w || !shape || !def || world < 0 || world >= (int)w->worlds.size())
        return fail(DBOX_ERR_INVALID, "dbox_fixture_create: bad arguments");
    HostWorld& hw0 = w->worlds[world];
    if (body < 0 || body >= (int)hw0.bs.size() || body_gone(hw0, body)) return fail(DBOX_ERR_INVALID, "dbox_fixture_create: no body %d", body);
    int rc = prepare_edit(w);
    if (rc) return rc;
    int idx = create_fixture(w->worlds[world], body, shape, def);
    if (idx < 0) return fail(DBOX_ERR_INVALID, "dbox_fixture_create: degenerate or unsupported shape");
    if (out_fixture) *out_fixture = idx;
    return DBOX_OK;
}

// the child edges of a b2ChainShape (b2chainshape.d: CreateChain / CreateLoop, GetChildEdge)
// as edge shape records, in child order
static ChainRec make_chain(const dbox_vec2* vertices, int count, bool loop, const dbox_vec2* prev, const dbox_vec2* next) {
    ChainRec c;
    c.v.assign(vertices, vertices + count);
    c.has_prev = prev != nullptr;
    c.has_next = next != nullptr;
    c.prev = prev ? *prev : dbox_vec2{0.0f, 0.0f};
    c.next = next ? *next : dbox_vec2{0.0f, 0.0f};
    if (loop) {
        c.v.push_back(vertices[0]);
        c.prev = c.v[c.v.size() - 2];
        c.next = c.v[1];
        c.has_prev = c.has_next = 1;
    }
    c.density = 0.0f;
    c.first = -1;
    c.dead = 0;
    return c;
}

static std::vector<dbox_shape_def> chain_children(const ChainRec& c) {
    const std::vector<dbox_vec2>& v = c.v;
    const bool hasPrev = c.has_prev != 0, hasNext = c.has_next != 0;
    const dbox_vec2 pv = c.prev, nv = c.next;
    const int m = (int)v.size();
    std::vector<dbox_shape_def> out;
    for (int i = 0; i + 1 < m; ++i) {
        dbox_shape_def e;
        memset(&e, 0, sizeof(e));
        e.kind = DBOX_SHAPE_EDGE;
        e.vertices[0] = v[i];
        e.vertices[1] = v[i + 1];
        int flags = 0;
        if (i > 0) { e.vertices[2] = v[i - 1]; flags |= 1; }
        else if (hasPrev) { e.vertices[2] = pv; flags |= 1; }
        if (i < m - 2) { e.vertices[3] = v[i + 2]; flags |= 2; }
        else if (hasNext) { e.vertices[3] = nv; flags |= 2; }
        e.count = flags;
        out.push_back(e);
    }
    return out;
}

int32_t dbox_fixture_create_chain(dbox_world* w, int32_t world, int32_t body, const dbox_vec2* vertices, int32_t count,
                                  int32_t loop, const dbox_vec2* prev_vertex, const dbox_vec2* next_vertex,
                                  const dbox_fixture_def* def, int32_t* out_first) {
    if (!w || !vertices || !def || world < 0 || world >= (int)w->worlds.size() || count < (loop ? 3 : 2))
        return fail(DBOX_ERR_INVALID, "dbox_fixture_create_chain: bad arguments");
    HostWorld& hw0 = w->worlds[world];
    if (body < 0 || body >= (int)hw0.bs.size() || body_gone(hw0, body)) return fail(DBOX_ERR_INVALID, "dbox_fixture_create_chain: no body %d", body);
    int rc = prepare_edit(w);
    if (rc) return rc;
    dbox_fixture_def d = *def;
    d.density = 0.0f;
    int first = -1;
    ChainRec c = make_chain(vertices, count, loop != 0, loop ? nullptr : prev_vertex, loop ? nullptr : next_vertex);
    for (const dbox_shape_def& e : chain_children(c)) {
        int idx = create_fixture(w->worlds[world], body, &e, &d);
        if (idx < 0) return fail(DBOX_ERR_INVALID, "dbox_fixture_create_chain: bad child edge");
        if (first < 0) first = idx;
    }
    c.density = def->density;
    c.first = first;
    w->worlds[world].chains.push_back(c);
    if (out_first) *out_first = first;
    return DBOX_OK;
}

// ---------------------------------------------------------------- destruction
// b2World.DestroyBody / DestroyJoint and b2Body.DestroyFixture on the host mirrors, between
// steps.  Destroyed bodies, fixtures and joints keep their indices as all-zero records (a
// fixture without a proxy, a joint of type -1); the contact list loses the destroyed
// contacts and keeps its order.  A body's contact list is its contacts newest first (the
// host list is oldest first), its joint list its joints newest first.
namespace {

void wake(dbox_body_state& s) {                                         // b2Body.SetAwake(true), b2body.d:827-846
    if ((s.flags & dg::kBodyAwake) == 0) {
        s.flags |= dg::kBodyAwake;
        s.sleep_time = 0.0f;
    }
}

// b2ContactManager.Destroy (b2contactmanager.d:183-246) with b2Contact.Destroy (b2contact.d:402-422)
void destroy_contact(HostWorld& hw, int ci, int world, std::vector<dbox_contact_event>& ev) {
    const dbox_contact_state c = hw.ct[ci];
    const dg::DFixture& fa = hw.fx[c.fixture_a];
    const dg::DFixture& fb = hw.fx[c.fixture_b];
    if (c.flags & dg::kContactTouching) {
        dbox_contact_event e;
        memset(&e, 0, sizeof(e));
        e.kind = DBOX_EVENT_END;
        e.world = world;
        e.fixture_a = c.fixture_a;
        e.fixture_b = c.fixture_b;
        e.point_count = c.point_count;
        ev.push_back(e);
    }
    if (c.point_count > 0 && !fa.sensor && !fb.sensor) {
        wake(hw.bs[fa.body]);
        wake(hw.bs[fb.body]);
    }
    hw.ct.erase(hw.ct.begin() + ci);
}

void destroy_joint(HostWorld& hw, int j) {                              // b2world.d:265-360
    dg::DJoint& d = hw.jt[j];
    const bool collide = d.collide_connected != 0;
    const int A = d.body_a, B = d.body_b;
    wake(hw.bs[A]);
    wake(hw.bs[B]);
    memset(&d, 0, sizeof(d));
    d.type = -1;
    d.body_a = A;
    d.body_b = B;
    if (!collide) {
        for (auto& c : hw.ct) {
            int a = hw.fx[c.fixture_a].body, b = hw.fx[c.fixture_b].body;
            if ((a == A && b == B) || (a == B && b == A)) c.flags |= dg::kContactFilter;
        }
    }
}

// the fixtures that are one reference fixture: a chain's child edges (child order), else fi
std::vector<int> fixture_group(const HostWorld& hw, int fi) {
    for (const ChainRec& c : hw.chains)
        if (!c.dead && fi >= c.first && fi < c.first + (int)c.v.size() - 1) {
            std::vector<int> g;
            for (int i = c.first; i < c.first + (int)c.v.size() - 1; ++i) g.push_back(i);
            return g;
        }
    return std::vector<int>(1, fi);
}

// b2Fixture.DestroyProxies (b2fixture.d:467-478) of a group, in child order
void free_proxies(HostWorld& hw, const std::vector<int>& g) {
    for (int fi : g) {
        dbox_proxy_state& p = hw.px[fi];
        if (p.proxy_id >= 0) hw.ids.destroy(p.proxy_id);
        memset(&p, 0, sizeof(p));
        p.proxy_id = -1;
    }
}

bool in_group(const std::vector<int>& g, int fi) { return std::find(g.begin(), g.end(), fi) != g.end(); }

void destroy_fixture(HostWorld& hw, int fi, int world, std::vector<dbox_contact_event>& ev) {   // b2body.d:179-247
    const int b = hw.fx[fi].body;
    const std::vector<int> g = fixture_group(hw, fi);
    std::vector<int>& list = hw.body_fix[b];
    list.erase(std::remove_if(list.begin(), list.end(), [&](int f) { return in_group(g, f); }), list.end());
    for (int ci = (int)hw.ct.size() - 1; ci >= 0; --ci) {
        const dbox_contact_state& c = hw.ct[ci];
        if (in_group(g, c.fixture_a) || in_group(g, c.fixture_b)) destroy_contact(hw, ci, world, ev);
    }
    if (hw.bs[b].flags & dg::kBodyActive) free_proxies(hw, g);
    for (ChainRec& c : hw.chains)
        if (c.first == g[0] && g.size() > 1) c.dead = 1;                // the chain is gone
    reset_mass(hw, b);
}

void destroy_body(HostWorld& hw, int b, int world, std::vector<dbox_contact_event>& ev) {      // b2world.d:105-193
    for (int j = (int)hw.jt.size() - 1; j >= 0; --j)
        if (hw.jt[j].type >= 0 && (hw.jt[j].body_a == b || hw.jt[j].body_b == b)) destroy_joint(hw, j);
    for (int ci = (int)hw.ct.size() - 1; ci >= 0; --ci) {
        const dbox_contact_state& c = hw.ct[ci];
        if (hw.fx[c.fixture_a].body == b || hw.fx[c.fixture_b].body == b) destroy_contact(hw, ci, world, ev);
    }
    std::vector<int> list = hw.body_fix[b];
    for (size_t k = 0; k < list.size();) {
        const std::vector<int> g = fixture_group(hw, list[k]);
        while (k < list.size() && in_group(g, list[k])) ++k;            // a chain is one fixture
        free_proxies(hw, g);
        for (ChainRec& c : hw.chains)
            if (c.first == g[0] && g.size() > 1) c.dead = 1;
    }
    hw.body_fix[b].clear();
    memset(&hw.bs[b], 0, sizeof(hw.bs[b]));
    if ((int)hw.body_dead.size() < (int)hw.bs.size()) hw.body_dead.resize(hw.bs.size(), 0);
    hw.body_dead[b] = 1;
}

int deliver_host_events(dbox_world* w, const std::vector<dbox_contact_event>& ev) {
    if (w->listener && !ev.empty()) w->listener(ev.data(), (int32_t)ev.size(), w->listener_user);
    return DBOX_OK;
}

}  // namespace

int32_t dbox_body_destroy(dbox_world* w, int32_t world, int32_t body) {
    if (!w || world < 0 || world >= (int)w->worlds.size()) return fail(DBOX_ERR_INVALID, "dbox_body_destroy: bad world");
    HostWorld& hw0 = w->worlds[world];
    if (body < 0 || body >= (int)hw0.bs.size() || body_gone(hw0, body))
        return fail(DBOX_ERR_INVALID, "dbox_body_destroy: no body %d", body);
    // b2World.DestroyBody destroys the body's joints newest first (b2world.d:115-131), so a
    // gear whose edge bodies (joint1's and joint2's B bodies) include this one goes before its
    // joints; only a body that carries a gear's joint but none of its edges would leave the
    // gear holding a destroyed joint
    for (const dg::DJoint& g : hw0.jt) {
        if (g.type != dg::kGearJoint || g.body_a == body || g.body_b == body) continue;
        for (int k : {g.joint1, g.joint2}) {
            const dg::DJoint& j = hw0.jt[k];
            if (j.body_a == body || j.body_b == body)
                return fail(DBOX_ERR_INVALID, "dbox_body_destroy: body %d carries a joint of a gear joint", body);
        }
    }
    int rc = prepare_edit(w);
    if (rc) return rc;
    std::vector<dbox_contact_event> ev;
    destroy_body(w->worlds[world], body, world, ev);
    return deliver_host_events(w, ev);
}

int32_t dbox_fixture_destroy(dbox_world* w, int32_t world, int32_t fixture) {
    if (!w || world < 0 || world >= (int)w->worlds.size()) return fail(DBOX_ERR_INVALID, "dbox_fixture_destroy: bad world");
    HostWorld& hw0 = w->worlds[world];
    if (fixture < 0 || fixture >= (int)hw0.fx.size() || body_gone(hw0, hw0.fx[fixture].body))
        return fail(DBOX_ERR_INVALID, "dbox_fixture_destroy: no fixture %d", fixture);
    const std::vector<int>& list = hw0.body_fix[hw0.fx[fixture].body];
    if (std::find(list.begin(), list.end(), fixture) == list.end())
        return fail(DBOX_ERR_INVALID, "dbox_fixture_destroy: fixture %d was destroyed", fixture);
    int rc = prepare_edit(w);
    if (rc) return rc;
    std::vector<dbox_contact_event> ev;
    destroy_fixture(w->worlds[world], fixture, world, ev);
    return deliver_host_events(w, ev);
}

int32_t dbox_joint_destroy(dbox_world* w, int32_t world, int32_t joint) {
    if (!w || world < 0 || world >= (int)w->worlds.size()) return fail(DBOX_ERR_INVALID, "dbox_joint_destroy: bad world");
    HostWorld& hw0 = w->worlds[world];
    if (joint < 0 || joint >= (int)hw0.jt.size() || hw0.jt[joint].type < 0)
        return fail(DBOX_ERR_INVALID, "dbox_joint_destroy: no joint %d", joint);
    for (const dg::DJoint& g : hw0.jt)
        if (g.type == dg::kGearJoint && (g.joint1 == joint || g.joint2 == joint))
            return fail(DBOX_ERR_INVALID, "dbox_joint_destroy: joint %d is used by a gear joint", joint);
    int rc = prepare_edit(w);
    if (rc) return rc;
    destroy_joint(w->worlds[world], joint);
    return DBOX_OK;
}

int32_t dbox_joint_create_revolute(dbox_world* w, int32_t world, const dbox_revolute_def* def, int32_t* out_joint) {
    if (!w || !def || world < 0 || world >= (int)w->worlds.size()) return fail(DBOX_ERR_INVALID, "dbox_joint_create_revolute: bad arguments");
    int rc = prepare_edit(w);
    if (rc) return rc;
    int idx = create_joint(w->worlds[world], def);
    if (idx < 0) return fail(DBOX_ERR_INVALID, "dbox_joint_create_revolute: bad bodies");
    if (out_joint) *out_joint = idx;
    return DBOX_OK;
}

// b2World.CreateJoint with a b2RopeJointDef (b2ropejoint.d:140-153)
int create_rope_joint(HostWorld& hw, const dbox_rope_def* d) {
    int nb = (int)hw.bs.size();
    if (d->body_a < 0 || d->body_a >= nb || d->body_b < 0 || d->body_b >= nb || d->body_a == d->body_b ||
        body_gone(hw, d->body_a) || body_gone(hw, d->body_b)) return -1;
    dg::DJoint j;
    memset(&j, 0, sizeof(j));
    j.type = dg::kRopeJoint;
    j.body_a = d->body_a;
    j.body_b = d->body_b;
    j.collide_connected = d->collide_connected ? 1 : 0;
    j.local_anchor_a = make_float2(d->local_anchor_a.x, d->local_anchor_a.y);
    j.local_anchor_b = make_float2(d->local_anchor_b.x, d->local_anchor_b.y);
    j.length = d->max_length;
    return link_joint(hw, j);
}

// b2World.CreateJoint with a b2WeldJointDef (b2weldjoint.d:107-119)
int create_weld_joint(HostWorld& hw, const dbox_weld_def* d) {
    int nb = (int)hw.bs.size();
    if (d->body_a < 0 || d->body_a >= nb || d->body_b < 0 || d->body_b >= nb || d->body_a == d->body_b ||
        body_gone(hw, d->body_a) || body_gone(hw, d->body_b)) return -1;
    dg::DJoint j;
    memset(&j, 0, sizeof(j));
    j.type = dg::kWeldJoint;
    j.body_a = d->body_a;
    j.body_b = d->body_b;
    j.collide_connected = d->collide_connected ? 1 : 0;
    j.local_anchor_a = make_float2(d->local_anchor_a.x, d->local_anchor_a.y);
    j.local_anchor_b = make_float2(d->local_anchor_b.x, d->local_anchor_b.y);
    j.reference_angle = d->reference_angle;
    j.frequency_hz = d->frequency_hz;
    j.damping_ratio = d->damping_ratio;
    return link_joint(hw, j);
}

// b2World.CreateJoint with a b2FrictionJointDef / b2MotorJointDef (b2frictionjoint.d:85-96, b2motorjoint.d:92-106)
int create_friction_joint(HostWorld& hw, const dbox_friction_def* d) {
    int nb = (int)hw.bs.size();
    if (d->body_a < 0 || d->body_a >= nb || d->body_b < 0 || d->body_b >= nb || d->body_a == d->body_b ||
        body_gone(hw, d->body_a) || body_gone(hw, d->body_b)) return -1;
    dg::DJoint j;
    memset(&j, 0, sizeof(j));
    j.type = dg::kFrictionJoint;
    j.body_a = d->body_a;
    j.body_b = d->body_b;
    j.collide_connected = d->collide_connected ? 1 : 0;
    j.local_anchor_a = make_float2(d->local_anchor_a.x, d->local_anchor_a.y);
    j.local_anchor_b = make_float2(d->local_anchor_b.x, d->local_anchor_b.y);
    j.max_force = d->max_force;
    j.max_torque = d->max_torque;
    return link_joint(hw, j);
}

int create_motor_joint(HostWorld& hw, const dbox_motor_def* d) {
    int nb = (int)hw.bs.size();
    if (d->body_a < 0 || d->body_a >= nb || d->body_b < 0 || d->body_b >= nb || d->body_a == d->body_b ||
        body_gone(hw, d->body_a) || body_gone(hw, d->body_b)) return -1;
    dg::DJoint j;
    memset(&j, 0, sizeof(j));
    j.type = dg::kMotorJoint;
    j.body_a = d->body_a;
    j.body_b = d->body_b;
    j.collide_connected = d->collide_connected ? 1 : 0;
    j.linear_offset = make_float2(d->linear_offset.x, d->linear_offset.y);
    j.angular_offset = d->angular_offset;
    j.max_force = d->max_force;
    j.max_torque = d->max_torque;
    j.correction_factor = d->correction_factor;
    return link_joint(hw, j);
}

// b2World.CreateJoint with a b2WheelJointDef (b2wheeljoint.d:110-139)
int create_wheel_joint(HostWorld& hw, const dbox_wheel_def* d) {
    int nb = (int)hw.bs.size();
    if (d->body_a < 0 || d->body_a >= nb || d->body_b < 0 || d->body_b >= nb || d->body_a == d->body_b ||
        body_gone(hw, d->body_a) || body_gone(hw, d->body_b)) return -1;
    dg::DJoint j;
    memset(&j, 0, sizeof(j));
    j.type = dg::kWheelJoint;
    j.body_a = d->body_a;
    j.body_b = d->body_b;
    j.collide_connected = d->collide_connected ? 1 : 0;
    j.local_anchor_a = make_float2(d->local_anchor_a.x, d->local_anchor_a.y);
    j.local_anchor_b = make_float2(d->local_anchor_b.x, d->local_anchor_b.y);
    j.local_axis_x = make_float2(d->local_axis_a.x, d->local_axis_a.y);
    j.local_axis_y = make_float2(-1.0f * d->local_axis_a.y, 1.0f * d->local_axis_a.x);   // b2Cross(1, x)
    j.enable_motor = d->enable_motor ? 1 : 0;
    j.max_motor_torque = d->max_motor_torque;
    j.motor_speed = d->motor_speed;
    j.frequency_hz = d->frequency_hz;
    j.damping_ratio = d->damping_ratio;
    return link_joint(hw, j);
}

// b2World.CreateJoint with a b2PrismaticJointDef (b2prismaticjoint.d:163-187): the axis is
// normalised as b2Vec2.Normalize does (b2math.d:160-175)
int create_prismatic_joint(HostWorld& hw, const dbox_prismatic_def* d) {
    int nb = (int)hw.bs.size();
    if (d->body_a < 0 || d->body_a >= nb || d->body_b < 0 || d->body_b >= nb || d->body_a == d->body_b ||
        body_gone(hw, d->body_a) || body_gone(hw, d->body_b)) return -1;
    dg::DJoint j;
    memset(&j, 0, sizeof(j));
    j.type = dg::kPrismaticJoint;
    j.body_a = d->body_a;
    j.body_b = d->body_b;
    j.collide_connected = d->collide_connected ? 1 : 0;
    j.local_anchor_a = make_float2(d->local_anchor_a.x, d->local_anchor_a.y);
    j.local_anchor_b = make_float2(d->local_anchor_b.x, d->local_anchor_b.y);
    float ax = d->local_axis_a.x, ay = d->local_axis_a.y;
    float len = sqrtf(ax * ax + ay * ay);
    if (!(len < FLT_EPSILON)) {
        float inv = 1.0f / len;
        ax *= inv;
        ay *= inv;
    }
    j.local_axis_x = make_float2(ax, ay);
    j.local_axis_y = make_float2(-1.0f * ay, 1.0f * ax);                 // b2Cross(1, x)
    j.reference_angle = d->reference_angle;
    j.enable_limit = d->enable_limit ? 1 : 0;
    j.lower_translation = d->lower_translation;
    j.upper_translation = d->upper_translation;
    j.enable_motor = d->enable_motor ? 1 : 0;
    j.max_motor_force = d->max_motor_force;
    j.motor_speed = d->motor_speed;
    return link_joint(hw, j);
}

// b2World.CreateJoint with a b2PulleyJointDef (b2pulleyjoint.d:116-131)
int create_pulley_joint(HostWorld& hw, const dbox_pulley_def* d) {
    int nb = (int)hw.bs.size();
    if (d->body_a < 0 || d->body_a >= nb || d->body_b < 0 || d->body_b >= nb || d->body_a == d->body_b ||
        body_gone(hw, d->body_a) || body_gone(hw, d->body_b)) return -1;
    dg::DJoint j;
    memset(&j, 0, sizeof(j));
    j.type = dg::kPulleyJoint;
    j.body_a = d->body_a;
    j.body_b = d->body_b;
    j.collide_connected = d->collide_connected ? 1 : 0;
    j.ground_a = make_float2(d->ground_anchor_a.x, d->ground_anchor_a.y);
    j.ground_b = make_float2(d->ground_anchor_b.x, d->ground_anchor_b.y);
    j.local_anchor_a = make_float2(d->local_anchor_a.x, d->local_anchor_a.y);
    j.local_anchor_b = make_float2(d->local_anchor_b.x, d->local_anchor_b.y);
    j.ratio = d->ratio;
    j.length_a = d->length_a;
    j.length_b = d->length_b;
    j.constant = d->length_a + d->ratio * d->length_b;
    return link_joint(hw, j);
}

// b2World.CreateJoint with a b2MouseJointDef (b2mousejoint.d:112-129): the local anchor is the
// target in body B's frame now (b2MulT(xf, v), b2math.d:743-751)
int create_mouse_joint(HostWorld& hw, const dbox_mouse_def* d) {
    int nb = (int)hw.bs.size();
    if (d->body_a < 0 || d->body_a >= nb || d->body_b < 0 || d->body_b >= nb || d->body_a == d->body_b ||
        body_gone(hw, d->body_a) || body_gone(hw, d->body_b)) return -1;
    dg::DJoint j;
    memset(&j, 0, sizeof(j));
    j.type = dg::kMouseJoint;
    j.body_a = d->body_a;
    j.body_b = d->body_b;
    j.collide_connected = d->collide_connected ? 1 : 0;
    j.target = make_float2(d->target.x, d->target.y);
    const float* xf = hw.bs[d->body_b].xf;
    float px = d->target.x - xf[0], py = d->target.y - xf[1];
    j.local_anchor_b = make_float2(xf[3] * px + xf[2] * py, -xf[2] * px + xf[3] * py);
    j.max_force = d->max_force;
    j.frequency_hz = d->frequency_hz;
    j.damping_ratio = d->damping_ratio;
    return link_joint(hw, j);
}

int32_t dbox_joint_create_pulley(dbox_world* w, int32_t world, const dbox_pulley_def* def, int32_t* out_joint) {
    if (!w || !def || world < 0 || world >= (int)w->worlds.size()) return fail(DBOX_ERR_INVALID, "dbox_joint_create_pulley: bad arguments");
    int rc = prepare_edit(w);
    if (rc) return rc;
    int idx = create_pulley_joint(w->worlds[world], def);
    if (idx < 0) return fail(DBOX_ERR_INVALID, "dbox_joint_create_pulley: bad bodies");
    if (out_joint) *out_joint = idx;
    return DBOX_OK;
}

// b2World.CreateJoint with a b2GearJointDef (b2gearjoint.d:83-168, b2world.d:196-261): the
// gear's own bodies are joint1's and joint2's B bodies; the definition's bodies only choose
// which contacts are flagged for filtering
int create_gear_joint(HostWorld& hw, const dbox_gear_def* d) {
    const int nb = (int)hw.bs.size(), nj = (int)hw.jt.size();
    if (d->body_a < 0 || d->body_a >= nb || d->body_b < 0 || d->body_b >= nb || d->body_a == d->body_b ||
        body_gone(hw, d->body_a) || body_gone(hw, d->body_b)) return -1;
    for (int k : {d->joint1, d->joint2})
        if (k < 0 || k >= nj || (hw.jt[k].type != dg::kRevoluteJoint && hw.jt[k].type != dg::kPrismaticJoint)) return -1;
    const dg::DJoint& j1 = hw.jt[d->joint1];
    const dg::DJoint& j2 = hw.jt[d->joint2];
    dg::DJoint j;
    memset(&j, 0, sizeof(j));
    j.type = dg::kGearJoint;
    j.collide_connected = d->collide_connected ? 1 : 0;
    j.joint1 = d->joint1;
    j.joint2 = d->joint2;
    j.type_a = j1.type;
    j.type_b = j2.type;
    // coordinate of a joint: its angle, or the slide along its axis (b2gearjoint.d:107-161)
    auto coordinate = [&](const dg::DJoint& jn, int body_other, int body_base, float2 anchor_base, float2 anchor_other,
                          float2 axis) {
        const dbox_body_state& o = hw.bs[body_other];
        const dbox_body_state& b = hw.bs[body_base];
        if (jn.type == dg::kRevoluteJoint) return (o.sweep[7] - b.sweep[7]) - jn.reference_angle;
        hg::Rot qo, qb;
        qo.s = o.xf[2]; qo.c = o.xf[3];
        qb.s = b.xf[2]; qb.c = b.xf[3];
        const hg::V2 m = hg::rmul(qo, hg::mk(anchor_other.x, anchor_other.y));
        const hg::V2 dp = hg::sub(hg::mk(o.xf[0], o.xf[1]), hg::mk(b.xf[0], b.xf[1]));
        const hg::V2 t = hg::add(m, dp);
        const hg::V2 p = hg::mk(qb.c * t.x + qb.s * t.y, -qb.s * t.x + qb.c * t.y);   // b2MulT(q, v)
        return hg::dot(hg::sub(p, hg::mk(anchor_base.x, anchor_base.y)), hg::mk(axis.x, axis.y));
    };
    j.body_c = j1.body_a;
    j.body_a = j1.body_b;
    j.local_anchor_c = j1.local_anchor_a;
    j.local_anchor_a = j1.local_anchor_b;
    j.reference_angle_a = j1.reference_angle;
    j.local_axis_c = j1.type == dg::kRevoluteJoint ? make_float2(0.0f, 0.0f) : j1.local_axis_x;
    const float coordinateA = coordinate(j1, j.body_a, j.body_c, j.local_anchor_c, j.local_anchor_a, j.local_axis_c);
    j.body_d = j2.body_a;
    j.body_b = j2.body_b;
    j.local_anchor_d = j2.local_anchor_a;
    j.local_anchor_b = j2.local_anchor_b;
    j.reference_angle_b = j2.reference_angle;
    j.local_axis_d = j2.type == dg::kRevoluteJoint ? make_float2(0.0f, 0.0f) : j2.local_axis_x;
    const float coordinateB = coordinate(j2, j.body_b, j.body_d, j.local_anchor_d, j.local_anchor_b, j.local_axis_d);
    j.ratio = d->ratio;
    j.constant = coordinateA + j.ratio * coordinateB;
    const int idx = (int)hw.jt.size();
    hw.jt.push_back(j);
    if (!j.collide_connected) {
        for (auto& c : hw.ct) {
            int A = hw.fx[c.fixture_a].body, B = hw.fx[c.fixture_b].body;
            if ((A == d->body_a && B == d->body_b) || (A == d->body_b && B == d->body_a)) c.flags |= dg::kContactFilter;
        }
    }
    return idx;
}

int32_t dbox_joint_create_gear(dbox_world* w, int32_t world, const dbox_gear_def* def, int32_t* out_joint) {
    if (!w || !def || world < 0 || world >= (int)w->worlds.size()) return fail(DBOX_ERR_INVALID, "dbox_joint_create_gear: bad arguments");
    int rc = prepare_edit(w);
    if (rc) return rc;
    int idx = create_gear_joint(w->worlds[world], def);
    if (idx < 0) return fail(DBOX_ERR_INVALID, "dbox_joint_create_gear: bad bodies or joints");
    if (out_joint) *out_joint = idx;
    return DBOX_OK;
}

int32_t dbox_joint_create_mouse(dbox_world* w, int32_t world, const dbox_mouse_def* def, int32_t* out_joint) {
    if (!w || !def || world < 0 || world >= (int)w->worlds.size()) return fail(DBOX_ERR_INVALID, "dbox_joint_create_mouse: bad arguments");
    int rc = prepare_edit(w);
    if (rc) return rc;
    int idx = create_mouse_joint(w->worlds[world], def);
    if (idx < 0) return fail(DBOX_ERR_INVALID, "dbox_joint_create_mouse: bad bodies");
    if (out_joint) *out_joint = idx;
    return DBOX_OK;
}

int32_t dbox_joint_set_mouse_target(dbox_world* w, int32_t world, int32_t joint, dbox_vec2 target) {
    if (!w || world < 0 || world >= (int)w->worlds.size()) return fail(DBOX_ERR_INVALID, "dbox_joint_set_mouse_target: bad world");
    int rc = prepare_edit(w);
    if (rc) return rc;
    HostWorld& hw = w->worlds[world];
    if (joint < 0 || joint >= (int)hw.jt.size() || hw.jt[joint].type != dg::kMouseJoint)
        return fail(DBOX_ERR_INVALID, "dbox_joint_set_mouse_target: not a mouse joint");
    dbox_body_state& b = hw.bs[hw.jt[joint].body_b];
    if ((b.flags & dg::kBodyAwake) == 0) { b.flags |= dg::kBodyAwake; b.sleep_time = 0.0f; }   // SetAwake(true)
    hw.jt[joint].target = make_float2(target.x, target.y);
    return DBOX_OK;
}

int32_t dbox_joint_create_prismatic(dbox_world* w, int32_t world, const dbox_prismatic_def* def, int32_t* out_joint) {
    if (!w || !def || world < 0 || world >= (int)w->worlds.size()) return fail(DBOX_ERR_INVALID, "dbox_joint_create_prismatic: bad arguments");
    int rc = prepare_edit(w);
    if (rc) return rc;
    int idx = create_prismatic_joint(w->worlds[world], def);
    if (idx < 0) return fail(DBOX_ERR_INVALID, "dbox_joint_create_prismatic: bad bodies");
    if (out_joint) *out_joint = idx;
    return DBOX_OK;
}

int32_t dbox_joint_create_wheel(dbox_world* w, int32_t world, const dbox_wheel_def* def, int32_t* out_joint) {
    if (!w || !def || world < 0 || world >= (int)w->worlds.size()) return fail(DBOX_ERR_INVALID, "dbox_joint_create_wheel: bad arguments");
    int rc = prepare_edit(w);
    if (rc) return rc;
    int idx = create_wheel_joint(w->worlds[world], def);
    if (idx < 0) return fail(DBOX_ERR_INVALID, "dbox_joint_create_wheel: bad bodies");
    if (out_joint) *out_joint = idx;
    return DBOX_OK;
}

int32_t dbox_joint_create_friction(dbox_world* w, int32_t world, const dbox_friction_def* def, int32_t* out_joint) {
    if (!w || !def || world < 0 || world >= (int)w->worlds.size()) return fail(DBOX_ERR_INVALID, "dbox_joint_create_friction: bad arguments");
    int rc = prepare_edit(w);
    if (rc) return rc;
    int idx = create_friction_joint(w->worlds[world], def);
    if (idx < 0) return fail(DBOX_ERR_INVALID, "dbox_joint_create_friction: bad bodies");
    if (out_joint) *out_joint = idx;
    return DBOX_OK;
}

int32_t dbox_joint_create_motor(dbox_world* w, int32_t world, const dbox_motor_def* def, int32_t* out_joint) {
    if (!w || !def || world < 0 || world >= (int)w->worlds.size()) return fail(DBOX_ERR_INVALID, "dbox_joint_create_motor: bad arguments");
    int rc = prepare_edit(w);
    if (rc) return rc;
    int idx = create_motor_joint(w->worlds[world], def);
    if (idx < 0) return fail(DBOX_ERR_INVALID, "dbox_joint_create_motor: bad bodies");
    if (out_joint) *out_joint = idx;
    return DBOX_OK;
}

int32_t dbox_joint_create_rope(dbox_world* w, int32_t world, const dbox_rope_def* def, int32_t* out_joint) {
    if (!w || !def || world < 0 || world >= (int)w->worlds.size()) return fail(DBOX_ERR_INVALID, "dbox_joint_create_rope: bad arguments");
    int rc = prepare_edit(w);
    if (rc) return rc;
    int idx = create_rope_joint(w->worlds[world], def);
    if (idx < 0) return fail(DBOX_ERR_INVALID, "dbox_joint_create_rope: bad bodies");
    if (out_joint) *out_joint = idx;
    return DBOX_OK;
}

int32_t dbox_joint_create_weld(dbox_world* w, int32_t world, const dbox_weld_def* def, int32_t* out_joint) {
    if (!w || !def || world < 0 || world >= (int)w->worlds.size()) return fail(DBOX_ERR_INVALID, "dbox_joint_create_weld: bad arguments");
    int rc = prepare_edit(w);
    if (rc) return rc;
    int idx = create_weld_joint(w->worlds[world], def);
    if (idx < 0) return fail(DBOX_ERR_INVALID, "dbox_joint_create_weld: bad bodies");
    if (out_joint) *out_joint = idx;
    return DBOX_OK;
}

int32_t dbox_joint_create_distance(dbox_world* w, int32_t world, const dbox_distance_def* def, int32_t* out_joint) {
    if (!w || !def || world < 0 || world >= (int)w->worlds.size()) return fail(DBOX_ERR_INVALID, "dbox_joint_create_distance: bad arguments");
    int rc = prepare_edit(w);
    if (rc) return rc;
    int idx = create_distance_joint(w->worlds[world], def);
    if (idx < 0) return fail(DBOX_ERR_INVALID, "dbox_joint_create_distance: bad bodies");
    if (out_joint) *out_joint = idx;
    return DBOX_OK;
}

int32_t dbox_scene_create(dbox_world* w, int32_t world, int32_t n_bodies, const dbox_body_def* bodies,
                          int32_t n_fixtures, const int32_t* fixture_body, const dbox_shape_def* shapes,
                          const dbox_fixture_def* fixtures, int32_t n_joints, const dbox_revolute_def* joints) {
    if (!w || world < 0 || world >= (int)w->worlds.size() || n_bodies < 0 || n_fixtures < 0 || n_joints < 0)
        return fail(DBOX_ERR_INVALID, "dbox_scene_create: bad arguments");
    if ((n_bodies && !bodies) || (n_fixtures && (!fixture_body || !shapes || !fixtures)) || (n_joints && !joints))
        return fail(DBOX_ERR_INVALID, "dbox_scene_create: null array");
    int rc = prepare_edit(w);
    if (rc) return rc;
    HostWorld& hw = w->worlds[world];
    int base = (int)hw.bs.size();
    hw.bs.reserve(base + n_bodies);
    hw.bst.reserve(base + n_bodies);
    for (int i = 0; i < n_bodies; ++i) {
        dbox_body_state s;
        dg::BodyStatic st;
        fill_body_state(bodies + i, &s, &st);
        hw.bs.push_back(s);
        hw.bst.push_back(st);
        hw.body_fix.emplace_back();
    }
    for (int i = 0; i < n_fixtures; ++i) {
        int b = base + fixture_body[i];
        if (fixture_body[i] < 0 || b >= (int)hw.bs.size()) return fail(DBOX_ERR_INVALID, "dbox_scene_create: fixture %d body", i);
        if (create_fixture(hw, b, shapes + i, fixtures + i) < 0)
            return fail(DBOX_ERR_INVALID, "dbox_scene_create: fixture %d degenerate or unsupported", i);
    }
    for (int i = 0; i < n_joints; ++i) {
        dbox_revolute_def d = joints[i];
        d.body_a += base;
        d.body_b += base;
        if (create_joint(hw, &d) < 0) return fail(DBOX_ERR_INVALID, "dbox_scene_create: joint %d bodies", i);
    }
    return DBOX_OK;
}

int32_t dbox_world_set_flags(dbox_world* w, int32_t warm_starting, int32_t continuous, int32_t sub_stepping,
                             int32_t allow_sleep, int32_t auto_clear_forces) {
    if (!w) return DBOX_ERR_INVALID;
    bool sleep_flag = allow_sleep != 0;
    if (sleep_flag != (w->allow_sleep != 0) && !sleep_flag) {
        // b2World.SetAllowSleeping(false) wakes every body (b2world.d:627-643)
        int rc = prepare_edit(w);
        if (rc) return rc;
        for (auto& hw : w->worlds)
            for (auto& b : hw.bs)
                if ((b.flags & dg::kBodyAwake) == 0) { b.flags |= dg::kBodyAwake; b.sleep_time = 0.0f; }
    }
    if ((auto_clear_forces != 0) != (w->autoclear != 0)) {
        int rc = prepare_edit(w);
        if (rc) return rc;
    }
    w->warm = warm_starting ? 1 : 0;
    w->continuous = continuous ? 1 : 0;
    w->substep = sub_stepping ? 1 : 0;
    w->allow_sleep = sleep_flag ? 1 : 0;
    w->autoclear = auto_clear_forces ? 1 : 0;
    if (w->graph) { cudaGraphExecDestroy(w->graph); w->graph = nullptr; }
    return DBOX_OK;
}

int32_t dbox_world_set_gravity(dbox_world* w, dbox_vec2 gravity) {
    if (!w) return DBOX_ERR_INVALID;
    w->gravity = make_float2(gravity.x, gravity.y);
    if (w->graph) { cudaGraphExecDestroy(w->graph); w->graph = nullptr; }
    return DBOX_OK;
}

int32_t dbox_world_set_listener(dbox_world* w, dbox_event_fn fn, void* user) {
    if (!w) return DBOX_ERR_INVALID;
    w->listener = fn;
    w->listener_user = user;
    if (fn && w->on_device) {
        int rc = alloc_mode_scratch(w);
        if (rc) return rc;
    }
    if (w->graph) { cudaGraphExecDestroy(w->graph); w->graph = nullptr; }
    if (w->tgraph) { cudaGraphExecDestroy(w->tgraph); w->tgraph = nullptr; }
    return DBOX_OK;
}

// b2Fixture.Refilter (b2fixture.d:140-180): flag the fixture's contacts for filtering and touch
// its proxies so that new pairs may be created
static void refilter(HostWorld& hw, int f) {
    for (auto& c : hw.ct)
        if (c.fixture_a == f || c.fixture_b == f) c.flags |= dg::kContactFilter;
    for (int g : fixture_group(hw, f))
        if (hw.px[g].proxy_id >= 0) hw.px[g].moved = 1;
}

static int edit_fixture(dbox_world* w, int32_t world, int32_t fixture, const char* what) {
    if (!w || world < 0 || world >= (int)w->worlds.size()) return fail(DBOX_ERR_INVALID, "%s: bad world", what);
    HostWorld& hw = w->worlds[world];
    if (fixture < 0 || fixture >= (int)hw.fx.size() || body_gone(hw, hw.fx[fixture].body))
        return fail(DBOX_ERR_INVALID, "%s: no fixture %d", what, fixture);
    const std::vector<int>& list = hw.body_fix[hw.fx[fixture].body];
    if (std::find(list.begin(), list.end(), fixture) == list.end())
        return fail(DBOX_ERR_INVALID, "%s: fixture %d was destroyed", what, fixture);
    return prepare_edit(w);
}

int32_t dbox_fixture_set_filter(dbox_world* w, int32_t world, int32_t fixture, uint16_t category_bits,
                                uint16_t mask_bits, int16_t group_index) {
    int rc = edit_fixture(w, world, fixture, "dbox_fixture_set_filter");
    if (rc) return rc;
    HostWorld& hw = w->worlds[world];
    for (int g : fixture_group(hw, fixture)) {                         // a chain's children share it
        hw.fx[g].filter = (uint32_t)category_bits | ((uint32_t)mask_bits << 16);
        hw.fx[g].group = group_index;
    }
    refilter(hw, fixture);
    return DBOX_OK;
}

int32_t dbox_fixture_set_filter_class(dbox_world* w, int32_t world, int32_t fixture, int32_t filter_class) {
    if (filter_class < 0 || filter_class > 63) return fail(DBOX_ERR_INVALID, "dbox_fixture_set_filter_class: class %d", filter_class);
    int rc = edit_fixture(w, world, fixture, "dbox_fixture_set_filter_class");
    if (rc) return rc;
    HostWorld& hw = w->worlds[world];
    for (int g : fixture_group(hw, fixture)) hw.fx[g].fclass = filter_class;
    refilter(hw, fixture);
    return DBOX_OK;
}

int32_t dbox_world_set_contact_filter(dbox_world* w, int32_t world, const uint64_t* table, int32_t with_default) {
    if (!w || world < 0 || world >= (int)w->worlds.size()) return fail(DBOX_ERR_INVALID, "dbox_world_set_contact_filter: bad world");
    if (table) {
        for (int a = 0; a < 64; ++a)
            for (int b = 0; b < 64; ++b)
                if (((table[a] >> b) & 1u) != ((table[b] >> a) & 1u))
                    return fail(DBOX_ERR_INVALID, "dbox_world_set_contact_filter: table not symmetric at (%d, %d)", a, b);
    }
    w->fmode.resize(w->worlds.size(), 0);
    w->ftab.resize(64 * w->worlds.size(), 0);
    w->fmode[world] = table ? (with_default ? 1 : 2) : 0;
    for (int a = 0; a < 64; ++a) w->ftab[64 * (size_t)world + a] = table ? table[a] : 0;
    w->filter_dirty = true;
    if (w->graph) { cudaGraphExecDestroy(w->graph); w->graph = nullptr; }
    if (w->tgraph) { cudaGraphExecDestroy(w->tgraph); w->tgraph = nullptr; }
    return DBOX_OK;
}

int32_t dbox_world_set_presolve(dbox_world* w, dbox_presolve_fn fn, void* user) {
    if (!w) return DBOX_ERR_INVALID;
    w->presolve = fn;
    w->presolve_user = user;
    if (fn && w->on_device) {
        int rc = alloc_mode_scratch(w);
        if (rc) return rc;
    }
    if (w->graph) { cudaGraphExecDestroy(w->graph); w->graph = nullptr; }
    if (w->tgraph) { cudaGraphExecDestroy(w->tgraph); w->tgraph = nullptr; }
    return DBOX_OK;
}

// The PreSolve window, after Collide and before Solve: the PRESOLVE events Collide recorded
// (per world, in contact-list order) name their contacts by fixture pair; the callback gets
// one record per call and may edit it; edited contacts are written back before the solve.
static int presolve_window(dbox_world* w) {
    const size_t W = w->worlds.size();
    std::vector<dg::WorldDyn> wd(W);
    CU(cudaStreamSynchronize(w->stream));
    CU(cudaMemcpy(wd.data(), w->d_wd.p, sizeof(dg::WorldDyn) * W, cudaMemcpyDeviceToHost));
    w->h_presolve.clear();
    std::vector<std::pair<size_t, size_t>> spans(W, {0, 0});         // records of each world
    std::vector<std::vector<dbox_contact_state>> cts(W);
    std::vector<std::vector<int>> where(W);                           // record -> contact slot
    std::vector<dbox_contact_event> ev;
    for (size_t i = 0; i < W; ++i) {
        const dg::WorldInfo& wi = w->wi[i];
        const int cnt = std::min(wd[i].ev_count, 4 * wi.contact_cap + 64);
        spans[i].first = w->h_presolve.size();
        if (cnt <= 0) { spans[i].second = spans[i].first; continue; }
        ev.resize(cnt);
        CU(cudaMemcpy(ev.data(), w->d_events.p + 4 * (size_t)wi.contact_start + 64 * i, sizeof(dbox_contact_event) * cnt,
                      cudaMemcpyDeviceToHost));
        bool any = false;
        for (const auto& e : ev) any |= e.kind == DBOX_EVENT_PRESOLVE;
        if (!any) { spans[i].second = spans[i].first; continue; }
        const int nct = wd[i].contact_count;
        cts[i].resize(nct);
        if (nct > 0)
            CU(cudaMemcpy(cts[i].data(), w->d_ct.p + wi.contact_start, sizeof(dbox_contact_state) * nct,
                          cudaMemcpyDeviceToHost));
        std::unordered_map<unsigned long long, int> slot;             // a fixture pair has one contact
        slot.reserve(2 * (size_t)nct);
        for (int k = 0; k < nct; ++k)
            slot[((unsigned long long)(unsigned)cts[i][k].fixture_a << 32) | (unsigned)cts[i][k].fixture_b] = k;
        for (const auto& e : ev) {
            if (e.kind != DBOX_EVENT_PRESOLVE) continue;
            const unsigned fa = (unsigned)(e.fixture_a + wi.fix_start), fb = (unsigned)(e.fixture_b + wi.fix_start);
            auto it = slot.find(((unsigned long long)fa << 32) | fb);
            if (it == slot.end()) return fail(DBOX_ERR_CUDA, "PreSolve window: no contact for fixtures %d, %d", e.fixture_a, e.fixture_b);
            const dbox_contact_state& c = cts[i][it->second];
            dbox_presolve_contact r;
            memset(&r, 0, sizeof(r));
            r.world = (int32_t)i;
            r.enabled = 1;
            r.friction = c.friction;
            r.restitution = c.restitution;
            r.tangent_speed = c.tangent_speed;
            r.contact = c;
            r.contact.fixture_a = e.fixture_a;
            r.contact.fixture_b = e.fixture_b;
            r.contact.flags &= ~(uint32_t)(dg::kContactUserOff | dg::kContactNew0 | dg::kContactNew1);
            w->h_presolve.push_back(r);
            where[i].push_back(it->second);
        }
        spans[i].second = w->h_presolve.size();
    }
    if (w->h_presolve.empty()) return DBOX_OK;
    w->presolve(w->h_presolve.data(), (int32_t)w->h_presolve.size(), w->presolve_user);
    for (size_t i = 0; i < W; ++i) {
        bool dirty = false;
        for (size_t r = spans[i].first; r < spans[i].second; ++r) {
            const dbox_presolve_contact& p = w->h_presolve[r];
            dbox_contact_state& c = cts[i][where[i][r - spans[i].first]];
            if (!p.enabled) { c.flags &= ~(uint32_t)dg::kContactEnabled; c.flags |= dg::kContactUserOff; dirty = true; }
            if (memcmp(&p.friction, &c.friction, 4) || memcmp(&p.restitution, &c.restitution, 4) ||
                memcmp(&p.tangent_speed, &c.tangent_speed, 4)) {
                c.friction = p.friction;
                c.restitution = p.restitution;
                c.tangent_speed = p.tangent_speed;
                dirty = true;
            }
        }
        if (dirty)
            CU(cudaMemcpyAsync(w->d_ct.p + w->wi[i].contact_start, cts[i].data(), sizeof(dbox_contact_state) * cts[i].size(),
                               cudaMemcpyHostToDevice, w->stream));
    }
    return DBOX_OK;
}

// the events of the last step, world by world, handed to the listener on this thread
static int deliver_events(dbox_world* w) {
    if (!w->listener || !w->d_events.p) return DBOX_OK;
    size_t W = w->worlds.size();
    std::vector<dg::WorldDyn> wd(W);
    CU(cudaStreamSynchronize(w->stream));
    CU(cudaMemcpy(wd.data(), w->d_wd.p, sizeof(dg::WorldDyn) * W, cudaMemcpyDeviceToHost));
    w->h_events.clear();
    for (size_t i = 0; i < W; ++i) {
        const dg::WorldInfo& wi = w->wi[i];
        int cnt = std::min(wd[i].ev_count, 4 * wi.contact_cap + 64);
        if (cnt <= 0) continue;
        size_t at = w->h_events.size();
        w->h_events.resize(at + cnt);
        CU(cudaMemcpy(&w->h_events[at], w->d_events.p + 4 * (size_t)wi.contact_start + 64 * i,
                      sizeof(dbox_contact_event) * cnt, cudaMemcpyDeviceToHost));
    }
    if (!w->h_events.empty()) w->listener(w->h_events.data(), (int32_t)w->h_events.size(), w->listener_user);
    return DBOX_OK;
}

// whole steps in one launch: asked for, and no large world (their steps span clusters) and no
// PreSolve window (the host acts between Collide and Solve)
static bool fused_ok(const dbox_world* w) { return w->fused_step && w->n_big == 0 && !w->presolve; }

int32_t dbox_world_step(dbox_world* w, float dt, int32_t velocity_iterations, int32_t position_iterations) {
    if (!w || velocity_iterations < 0 || position_iterations < 0) return fail(DBOX_ERR_INVALID, "dbox_world_step: bad arguments");
    int rc = ensure_device(w);
    if (rc) return rc;
    if (!w->events_made) {
        for (auto& e : w->ev) CU(cudaEventCreate(&e));
        w->events_made = true;
    }
    dg::Ctx x = make_ctx(w, dt, velocity_iterations, position_iterations);
    CU(cudaEventRecord(w->ev[0], w->stream));
    int launches = 0;
    int err;
    if (w->presolve) {                      // Collide, the host's PreSolve window, then Solve
        err = dbox_launch_collide(&x, w->stream);
        if (!err) {
            rc = presolve_window(w);
            if (rc) return rc;
            err = dbox_launch_solve(&x, w->stream, &launches);
        }
    } else if (fused_ok(w)) {
        x.steps = 1;
        err = dbox_launch_steps_fused(&x, w->stream, &launches);
    } else {
        err = dbox_launch_step(&x, w->stream, &launches);
    }
    if (err) return fail(DBOX_ERR_CUDA, "kernel launch failed: %s", cudaGetErrorString((cudaError_t)err));
    CU(cudaEventRecord(w->ev[1], w->stream));
    rc = check_status(w);
    float ms = 0.0f;
    cudaEventElapsedTime(&ms, w->ev[0], w->ev[1]);
    memset(&w->profile, 0, sizeof(w->profile));
    w->profile.step = ms;
    w->last_launches = launches;
    if (!rc) rc = deliver_events(w);
    return rc;
}

int32_t dbox_world_step_n(dbox_world* w, float dt, int32_t velocity_iterations, int32_t position_iterations,
                          int32_t steps) {
    if (!w || steps < 0 || velocity_iterations < 0 || position_iterations < 0)
        return fail(DBOX_ERR_INVALID, "dbox_world_step_n: bad arguments");
    int rc = ensure_device(w);
    if (rc) return rc;
    if (w->listener || w->presolve) {       // events are delivered / PreSolve is called in every step
        for (int i = 0; i < steps && !rc; ++i) rc = dbox_world_step(w, dt, velocity_iterations, position_iterations);
        return rc;
    }
    if (fused_ok(w)) {                      // every step of every world in one launch
        if (steps == 0) return DBOX_OK;
        dg::Ctx x = make_ctx(w, dt, velocity_iterations, position_iterations);
        x.steps = steps;
        int launches = 0;
        int err = dbox_launch_steps_fused(&x, w->stream, &launches);
        if (err) return fail(DBOX_ERR_CUDA, "kernel launch failed: %s", cudaGetErrorString((cudaError_t)err));
        w->last_launches = launches;
        return check_status(w);
    }
    int flags = w->warm | (w->continuous << 1) | (w->substep << 2) | (w->allow_sleep << 3) | (w->autoclear << 4);
    if (!w->graph || w->g_dt != dt || w->g_vi != velocity_iterations || w->g_pi != position_iterations ||
        w->graph_flags != flags) {
        if (w->graph) { cudaGraphExecDestroy(w->graph); w->graph = nullptr; }
        dg::Ctx x = make_ctx(w, dt, velocity_iterations, position_iterations);
        cudaGraph_t g;
        CU(cudaStreamBeginCapture(w->stream, cudaStreamCaptureModeThreadLocal));
        int launches = 0;
        int err = dbox_launch_step(&x, w->stream, &launches);
        cudaError_t ce = cudaStreamEndCapture(w->stream, &g);
        if (err || ce != cudaSuccess) return fail(DBOX_ERR_CUDA, "graph capture failed");
        CU(cudaGraphInstantiate(&w->graph, g, 0));
        cudaGraphDestroy(g);
        w->g_dt = dt; w->g_vi = velocity_iterations; w->g_pi = position_iterations; w->graph_flags = flags;
        w->g_launches = launches;
    }
    for (int i = 0; i < steps; ++i) CU(cudaGraphLaunch(w->graph, w->stream));
    w->last_launches = w->g_launches * steps;
    return check_status(w);
}

int32_t dbox_world_step_n_timed(dbox_world* w, float dt, int32_t velocity_iterations, int32_t position_iterations,
                                int32_t steps, float* total_ms, float* phase_ms) {
    if (!w || steps < 1 || velocity_iterations < 0 || position_iterations < 0)
        return fail(DBOX_ERR_INVALID, "dbox_world_step_n_timed: bad arguments");
    if (w->presolve) return fail(DBOX_ERR_UNSUPPORTED, "dbox_world_step_n_timed: a PreSolve window needs dbox_world_step");
    int rc = ensure_device(w);
    if (rc) return rc;
    if (fused_ok(w)) {                      // one launch: the whole step is phase 1
        if (w->tev.size() < 2) {
            for (auto& e : w->tev) cudaEventDestroy(e);
            w->tev.assign(2, nullptr);
            for (auto& e : w->tev) CU(cudaEventCreate(&e));
            if (w->tgraph) { cudaGraphExecDestroy(w->tgraph); w->tgraph = nullptr; }
        }
        dg::Ctx x = make_ctx(w, dt, velocity_iterations, position_iterations);
        x.steps = steps;
        int launches = 0;
        CU(cudaEventRecord(w->tev[0], w->stream));
        int err = dbox_launch_steps_fused(&x, w->stream, &launches);
        CU(cudaEventRecord(w->tev[1], w->stream));
        if (err) return fail(DBOX_ERR_CUDA, "kernel launch failed: %s", cudaGetErrorString((cudaError_t)err));
        w->last_launches = launches;
        rc = check_status(w);
        float tot = 0.0f;
        CU(cudaEventElapsedTime(&tot, w->tev[0], w->tev[1]));
        if (total_ms) *total_ms = tot;
        if (phase_ms) { phase_ms[0] = 0.0f; phase_ms[1] = tot; phase_ms[2] = 0.0f; }
        memset(&w->profile, 0, sizeof(w->profile));
        w->profile.step = tot / steps;
        return rc;
    }
    int flags = w->warm | (w->continuous << 1) | (w->substep << 2) | (w->allow_sleep << 3) | (w->autoclear << 4);
    if (!w->tgraph || w->t_steps != steps || w->t_dt != dt || w->t_vi != velocity_iterations ||
        w->t_pi != position_iterations || w->t_flags != flags) {
        if (w->tgraph) { cudaGraphExecDestroy(w->tgraph); w->tgraph = nullptr; }
        for (auto& e : w->tev) cudaEventDestroy(e);
        w->tev.assign(4 * (size_t)steps, nullptr);
        for (auto& e : w->tev) CU(cudaEventCreate(&e));
        dg::Ctx x = make_ctx(w, dt, velocity_iterations, position_iterations);
        cudaGraph_t g;
        CU(cudaStreamBeginCapture(w->stream, cudaStreamCaptureModeThreadLocal));
        int launches = 0, err = 0;
        for (int i = 0; i < steps && !err; ++i) err = dbox_launch_step_ev(&x, w->stream, &launches, &w->tev[4 * i]);
        cudaError_t ce = cudaStreamEndCapture(w->stream, &g);
        if (err || ce != cudaSuccess) return fail(DBOX_ERR_CUDA, "timed graph capture failed");
        CU(cudaGraphInstantiate(&w->tgraph, g, 0));
        cudaGraphDestroy(g);
        w->t_steps = steps; w->t_dt = dt; w->t_vi = velocity_iterations; w->t_pi = position_iterations;
        w->t_flags = flags;
        w->t_launches = launches * steps;
    }
    CU(cudaGraphLaunch(w->tgraph, w->stream));
    w->last_launches = w->t_launches;
    rc = check_status(w);
    float tot = 0.0f, ph[3] = {0.0f, 0.0f, 0.0f};
    CU(cudaEventElapsedTime(&tot, w->tev[0], w->tev[4 * (size_t)steps - 1]));
    for (int i = 0; i < steps; ++i)
        for (int p = 0; p < 3; ++p) {
            float ms = 0.0f;
            CU(cudaEventElapsedTime(&ms, w->tev[4 * i + p], w->tev[4 * i + p + 1]));
            ph[p] += ms;
        }
    if (total_ms) *total_ms = tot;
    if (phase_ms) { phase_ms[0] = ph[0]; phase_ms[1] = ph[1]; phase_ms[2] = ph[2]; }
    memset(&w->profile, 0, sizeof(w->profile));
    w->profile.step = tot / steps;
    w->profile.collide = ph[0] / steps;
    w->profile.solve = ph[1] / steps;
    w->profile.solve_toi = ph[2] / steps;
    return rc;
}

int32_t dbox_world_get_counters(dbox_world* w, unsigned long long* out) {
    if (!w || !out) return DBOX_ERR_INVALID;
    memset(out, 0, sizeof(unsigned long long) * 8);
    if (!w->on_device) return DBOX_OK;
    int W = (int)w->worlds.size();
    std::vector<dg::WorldDyn> wd(W);
    CU(cudaStreamSynchronize(w->stream));
    CU(cudaMemcpy(wd.data(), w->d_wd.p, sizeof(dg::WorldDyn) * W, cudaMemcpyDeviceToHost));
    for (auto& d : wd) {
        out[0] += d.acc_isl_bodies; out[1] += d.acc_isl_contacts; out[2] += d.acc_vsolve; out[3] += d.acc_psolve;
        out[4] += d.acc_contacts; out[5] += d.acc_toi_events; out[6] += d.acc_steps; out[7] += d.acc_pairs;
    }
    return DBOX_OK;
}

int32_t dbox_world_apply_forces(dbox_world* w, const float* force_torque) {
    if (!w || !force_torque) return fail(DBOX_ERR_INVALID, "dbox_world_apply_forces: bad arguments");
    int rc = ensure_device(w);
    if (rc) return rc;
    int n = w->total_bodies;
    if (n == 0) return DBOX_OK;
    CU(cudaMemcpyAsync(w->d_io.p, force_torque, sizeof(float) * 3 * (size_t)n, cudaMemcpyHostToDevice, w->stream));
    int err = dbox_launch_apply_forces(n, w->d_bs.p, w->d_io.p, w->stream);
    if (err) return fail(DBOX_ERR_CUDA, "apply forces launch: %s", cudaGetErrorString((cudaError_t)err));
    return DBOX_OK;
}

int32_t dbox_world_get_transforms(dbox_world* w, float* xya) {
    if (!w || !xya) return fail(DBOX_ERR_INVALID, "dbox_world_get_transforms: bad arguments");
    int rc = ensure_device(w);
    if (rc) return rc;
    int n = w->total_bodies;
    if (n == 0) return DBOX_OK;
    int err = dbox_launch_gather_transforms(n, w->d_bs.p, w->d_io.p, w->stream);
    if (err) return fail(DBOX_ERR_CUDA, "gather launch: %s", cudaGetErrorString((cudaError_t)err));
    CU(cudaMemcpyAsync(xya, w->d_io.p, sizeof(float) * 3 * (size_t)n, cudaMemcpyDeviceToHost, w->stream));
    CU(cudaStreamSynchronize(w->stream));
    return DBOX_OK;
}

int32_t dbox_world_set_warmstart(dbox_world* w, int32_t mode, dbox_mlp* model, int32_t sample_capacity) {
    if (!w || mode < 0 || mode > 3) return fail(DBOX_ERR_INVALID, "dbox_world_set_warmstart: bad mode");
    if (mode == 2 && !model) return fail(DBOX_ERR_INVALID, "dbox_world_set_warmstart: learned mode needs a model");
    if (mode == 1 && sample_capacity <= 0) return fail(DBOX_ERR_INVALID, "dbox_world_set_warmstart: sample capacity must be > 0");
    w->ws_mode = mode;
    w->mlp = mode == 2 ? model : nullptr;
    if (mode != 3) w->start_src = nullptr;
    if (mode == 1 && sample_capacity != w->sample_cap) {
        w->d_samples.free();
        w->d_sample_count.free();
        if (w->d_samples.alloc((size_t)dg::kSampleFloats * sample_capacity) || w->d_sample_count.alloc(1))
            return fail(DBOX_ERR_CUDA, "device allocation failed (%d samples)", sample_capacity);
        w->sample_cap = sample_capacity;
        CU(cudaMemset(w->d_sample_count.p, 0, sizeof(unsigned)));
    }
    if (w->on_device) {
        int rc = alloc_mode_scratch(w);
        if (rc) return rc;
    }
    if (w->graph) { cudaGraphExecDestroy(w->graph); w->graph = nullptr; }
    if (w->tgraph) { cudaGraphExecDestroy(w->tgraph); w->tgraph = nullptr; }
    return DBOX_OK;
}

// the two handles hold the same worlds laid out the same way on the device
static bool same_layout(const dbox_world* a, const dbox_world* b) {
    if (a->wi.size() != b->wi.size() || !a->on_device || !b->on_device || a->dirty || b->dirty) return false;
    return a->wi.empty() || memcmp(a->wi.data(), b->wi.data(), sizeof(dg::WorldInfo) * a->wi.size()) == 0;
}

int32_t dbox_world_set_start_source(dbox_world* w, dbox_world* src) {
    if (!w || !src || w == src || w->ws_mode != 3) return fail(DBOX_ERR_INVALID, "dbox_world_set_start_source: bad arguments");
    int rc = ensure_device(w);
    if (!rc) rc = ensure_device(src);
    if (rc) return rc;
    if (!same_layout(w, src)) return fail(DBOX_ERR_INVALID, "dbox_world_set_start_source: the handles' worlds differ");
    w->start_src = src;
    if (w->graph) { cudaGraphExecDestroy(w->graph); w->graph = nullptr; }
    if (w->tgraph) { cudaGraphExecDestroy(w->tgraph); w->tgraph = nullptr; }
    return DBOX_OK;
}

int32_t dbox_world_copy_state(dbox_world* dst, dbox_world* src) {
    if (!dst || !src || dst == src) return fail(DBOX_ERR_INVALID, "dbox_world_copy_state: bad arguments");
    int rc = ensure_device(dst);
    if (!rc) rc = ensure_device(src);
    if (rc) return rc;
    if (!same_layout(dst, src)) return fail(DBOX_ERR_INVALID, "dbox_world_copy_state: the handles' worlds differ");
    CU(cudaStreamSynchronize(src->stream));
    CU(cudaStreamSynchronize(dst->stream));
    auto cp = [&](void* d, const void* s, size_t bytes) -> cudaError_t {
        return bytes ? cudaMemcpyAsync(d, s, bytes, cudaMemcpyDeviceToDevice, dst->stream) : cudaSuccess;
    };
    CU(cp(dst->d_wd.p, src->d_wd.p, sizeof(dg::WorldDyn) * src->wi.size()));
    CU(cp(dst->d_bs.p, src->d_bs.p, sizeof(dbox_body_state) * src->d_bs.n));
    CU(cp(dst->d_px.p, src->d_px.p, sizeof(dbox_proxy_state) * src->d_px.n));
    CU(cp(dst->d_jt.p, src->d_jt.p, sizeof(dg::DJoint) * src->d_jt.n));
    CU(cp(dst->d_ct.p, src->d_ct.p, sizeof(dbox_contact_state) * src->d_ct.n));
    CU(cp(dst->d_hash.p, src->d_hash.p, sizeof(unsigned long long) * src->d_hash.n));
    CU(cudaStreamSynchronize(dst->stream));
    dst->mirrors_fresh = false;
    ++dst->gen;
    return DBOX_OK;
}

int32_t dbox_world_sample_count(dbox_world* w, int32_t* count) {
    if (!w || !count) return fail(DBOX_ERR_INVALID, "dbox_world_sample_count: null argument");
    unsigned c = 0;
    if (w->d_sample_count.p) {
        CU(cudaStreamSynchronize(w->stream));
        CU(cudaMemcpy(&c, w->d_sample_count.p, sizeof(unsigned), cudaMemcpyDeviceToHost));
    }
    *count = (int32_t)std::min<unsigned>(c, (unsigned)w->sample_cap);
    return DBOX_OK;
}

int32_t dbox_world_get_samples(dbox_world* w, int32_t offset, int32_t n, float* rows) {
    if (!w || !rows || offset < 0 || n < 0 || offset + n > w->sample_cap)
        return fail(DBOX_ERR_INVALID, "dbox_world_get_samples: bad range");
    if (n == 0) return DBOX_OK;
    CU(cudaStreamSynchronize(w->stream));
    CU(cudaMemcpy(rows, w->d_samples.p + (size_t)dg::kSampleFloats * offset, sizeof(float) * dg::kSampleFloats * n,
                  cudaMemcpyDeviceToHost));
    return DBOX_OK;
}

int32_t dbox_world_clear_samples(dbox_world* w) {
    if (!w) return DBOX_ERR_INVALID;
    if (w->d_sample_count.p) CU(cudaMemsetAsync(w->d_sample_count.p, 0, sizeof(unsigned), w->stream));
    return DBOX_OK;
}

int32_t dbox_mlp_train_world(dbox_mlp* m, dbox_world* w, int32_t epochs, int32_t batch, float lr, uint64_t seed,
                             float* epoch_loss) {
    if (!m || !w) return fail(DBOX_ERR_INVALID, "dbox_mlp_train_world: null argument");
    int32_t n = 0;
    int rc = dbox_world_sample_count(w, &n);
    if (rc) return rc;
    if (n <= 0) return fail(DBOX_ERR_INVALID, "dbox_mlp_train_world: the world holds no samples");
    return dbox_mlp_train_device(m, n, w->d_samples.p, epochs, batch, lr, seed, epoch_loss);
}

int32_t dbox_world_set_wait_limit(dbox_world* w, int32_t polls) {
    if (!w || polls < 0) return fail(DBOX_ERR_INVALID, "dbox_world_set_wait_limit: bad arguments");
    w->wait_polls = polls < (1 << 20) ? polls : (1 << 20);
    if (w->graph) { cudaGraphExecDestroy(w->graph); w->graph = nullptr; }
    if (w->tgraph) { cudaGraphExecDestroy(w->tgraph); w->tgraph = nullptr; }
    return DBOX_OK;
}

int32_t dbox_world_set_fused_step(dbox_world* w, int32_t enable) {
    if (!w || enable < 0 || enable > 1) return fail(DBOX_ERR_INVALID, "dbox_world_set_fused_step: bad arguments");
    w->fused_step = enable;
    return DBOX_OK;
}

int32_t dbox_world_get_fused_step(dbox_world* w, int32_t* enable) {
    if (!w || !enable) return fail(DBOX_ERR_INVALID, "dbox_world_get_fused_step: bad arguments");
    *enable = w->fused_step;
    return DBOX_OK;
}

int32_t dbox_world_get_island_solver(dbox_world* w, int32_t* mode) {
    if (!w || !mode) return fail(DBOX_ERR_INVALID, "dbox_world_get_island_solver: bad arguments");
    *mode = w->island_solver;
    return DBOX_OK;
}

int32_t dbox_world_set_island_solver(dbox_world* w, int32_t mode) {
    if (!w || mode < 0 || mode > 1) return fail(DBOX_ERR_INVALID, "dbox_world_set_island_solver: bad arguments");
    w->island_solver = mode;
    if (w->graph) { cudaGraphExecDestroy(w->graph); w->graph = nullptr; }
    if (w->tgraph) { cudaGraphExecDestroy(w->tgraph); w->tgraph = nullptr; }
    return DBOX_OK;
}

int32_t dbox_world_set_measure(dbox_world* w, int32_t enable) {
    if (!w) return DBOX_ERR_INVALID;
    w->measure = enable ? 1 : 0;
    if (w->on_device) {
        int rc = alloc_mode_scratch(w);
        if (rc) return rc;
    }
    if (w->graph) { cudaGraphExecDestroy(w->graph); w->graph = nullptr; }
    if (w->tgraph) { cudaGraphExecDestroy(w->tgraph); w->tgraph = nullptr; }
    return DBOX_OK;
}

int32_t dbox_world_get_quality(dbox_world* w, float* out) {
    if (!w || !out) return fail(DBOX_ERR_INVALID, "dbox_world_get_quality: null argument");
    if (!w->on_device) return fail(DBOX_ERR_INVALID, "dbox_world_get_quality: no step taken");
    size_t W = w->worlds.size();
    std::vector<dg::WorldDyn> wd(W);
    CU(cudaStreamSynchronize(w->stream));
    CU(cudaMemcpy(wd.data(), w->d_wd.p, sizeof(dg::WorldDyn) * W, cudaMemcpyDeviceToHost));
    for (size_t i = 0; i < W; ++i) {
        out[4 * i] = wd[i].q_sumsq;
        out[4 * i + 1] = wd[i].q_max;
        out[4 * i + 2] = (float)wd[i].q_points;
        out[4 * i + 3] = wd[i].q_minsep;
    }
    return DBOX_OK;
}

int32_t dbox_world_set_mapping(dbox_world* w, int32_t warps_per_block, int32_t body_budget) {
    return dbox_world_set_mapping_isolated(w, warps_per_block, body_budget, 0);
}

int32_t dbox_world_set_mapping_isolated(dbox_world* w, int32_t warps_per_block, int32_t body_budget, int32_t isolate) {
    if (!w || !(warps_per_block == 1 || warps_per_block == 2 || warps_per_block == dg::kSolveWarps) || body_budget < 0 ||
        isolate < 0)
        return fail(DBOX_ERR_INVALID, "dbox_world_set_mapping: warps per block must be 1, 2 or %d", dg::kSolveWarps);
    w->solve_queue_mode = 0;
    w->solve_wpb = warps_per_block;
    w->solve_budget = body_budget;
    w->solve_isolate = isolate;
    if (w->on_device) {
        int rc = pack_solve_slots(w);
        if (rc) return rc;
    }
    if (w->graph) { cudaGraphExecDestroy(w->graph); w->graph = nullptr; }
    if (w->tgraph) { cudaGraphExecDestroy(w->tgraph); w->tgraph = nullptr; }
    return DBOX_OK;
}

int32_t dbox_world_set_mapping_queue(dbox_world* w, int32_t heavy, int32_t exclusive, int32_t blocks_per_sm) {
    if (!w || heavy < 0 || blocks_per_sm < 0)
        return fail(DBOX_ERR_INVALID, "dbox_world_set_mapping_queue: bad arguments");
    w->solve_queue_mode = 1;
    w->solve_heavy = heavy;
    w->solve_exclusive = exclusive ? 1 : 0;
    w->solve_bps = blocks_per_sm;
    if (w->on_device) {
        int rc = pack_solve_slots(w);
        if (rc) return rc;
    }
    if (w->graph) { cudaGraphExecDestroy(w->graph); w->graph = nullptr; }
    if (w->tgraph) { cudaGraphExecDestroy(w->tgraph); w->tgraph = nullptr; }
    return DBOX_OK;
}

int32_t dbox_world_set_world_costs(dbox_world* w, const float* cost) {
    if (!w) return DBOX_ERR_INVALID;
    if (cost) w->world_cost.assign(cost, cost + w->worlds.size());
    else w->world_cost.clear();
    if (w->on_device && w->solve_queue_mode) {
        int rc = pack_solve_slots(w);
        if (rc) return rc;
    }
    return DBOX_OK;
}

int32_t dbox_world_get_world_costs(dbox_world* w, float* out) {
    if (!w || !out) return DBOX_ERR_INVALID;
    for (size_t i = 0; i < w->worlds.size(); ++i)
        out[i] = i < w->world_cost.size() ? w->world_cost[i] : (float)w->worlds[i].bs.size();
    return DBOX_OK;
}

int32_t dbox_world_autotune(dbox_world* w, float dt, int32_t velocity_iterations, int32_t position_iterations,
                            int32_t steps, int32_t* choice) {
    if (!w || steps < 1) return fail(DBOX_ERR_INVALID, "dbox_world_autotune: bad arguments");
    int rc = ensure_device(w);
    if (rc) return rc;
    if (w->nsm <= 0) {
        int dev = 0;
        CU(cudaGetDevice(&dev));
        CU(cudaDeviceGetAttribute(&w->nsm, cudaDevAttrMultiProcessorCount, dev));
    }
    // per-world costs for the queue order: the warp time of each world in one profiled step
    {
        const int was = w->profiling;
        rc = dbox_world_set_phase_profile(w, 1);
        if (!rc) rc = dbox_world_step_n(w, dt, velocity_iterations, position_iterations, 1);
        std::vector<unsigned long long> prof((size_t)dg::kProfSlots * w->worlds.size());
        if (!rc) rc = dbox_world_get_phase_profile(w, prof.data());
        int rc2 = dbox_world_set_phase_profile(w, was);
        if (rc) return rc;
        if (rc2) return rc2;
        std::vector<float> cost(w->worlds.size());
        for (size_t i = 0; i < cost.size(); ++i) {
            unsigned long long g0 = prof[dg::kProfSlots * i + 25], g1 = prof[dg::kProfSlots * i + 26];
            cost[i] = g1 > g0 ? (float)(g1 - g0) : 0.0f;
        }
        w->world_cost = cost;
    }
    // candidates: {queue, warps per block or heavy worlds, body budget or exclusive, isolated}
    const int S = w->nsm;
    const int cand[][4] = {{0, dg::kSolveWarps, 0, 0}, {0, 2, 0, 0}, {0, 1, 0, 0}, {0, dg::kSolveWarps, 2048, 0},
                           {0, 2, 2048, 0}, {0, dg::kSolveWarps, 2048, 152}, {0, dg::kSolveWarps, 2048, 304},
                           {1, 0, 0, 0}, {1, S, 0, 0}, {1, S / 2, 1, 0}};
    const int ncand = (int)(sizeof(cand) / sizeof(cand[0]));
    auto apply = [&](int c) {
        if (cand[c][0]) return dbox_world_set_mapping_queue(w, cand[c][1], cand[c][2], 0);
        return dbox_world_set_mapping_isolated(w, cand[c][1], cand[c][2], cand[c][3]);
    };
    cudaEvent_t e0, e1;
    CU(cudaEventCreate(&e0));
    CU(cudaEventCreate(&e1));
    float best = 3.4e38f;
    int bi = 0;
    for (int round = 0; round < 2 && !rc; ++round) {            // two rounds: the state drifts between trials
        for (int c = 0; c < ncand && !rc; ++c) {
            rc = apply(c);
            if (!rc) rc = dbox_world_step_n(w, dt, velocity_iterations, position_iterations, 1);   // builds the graph
            if (rc) break;
            CU(cudaEventRecord(e0, w->stream));
            rc = dbox_world_step_n(w, dt, velocity_iterations, position_iterations, steps);
            CU(cudaEventRecord(e1, w->stream));
            CU(cudaEventSynchronize(e1));
            float ms = 0.0f;
            cudaEventElapsedTime(&ms, e0, e1);
            if (round == 1 && ms < best) { best = ms; bi = c; }
        }
    }
    if (rc) { cudaEventDestroy(e0); cudaEventDestroy(e1); return rc; }
    rc = apply(bi);
    // large worlds: their Solve on a block or on a warp, timed the same way under the mapping kept
    if (!rc && w->n_big > 0) {
        float tbest[2] = {3.4e38f, 3.4e38f};
        for (int round = 0; round < 2 && !rc; ++round)
            for (int mode = 0; mode < 2 && !rc; ++mode) {
                rc = dbox_world_set_island_solver(w, mode);
                if (!rc) rc = dbox_world_step_n(w, dt, velocity_iterations, position_iterations, 1);
                if (rc) break;
                CU(cudaEventRecord(e0, w->stream));
                rc = dbox_world_step_n(w, dt, velocity_iterations, position_iterations, steps);
                CU(cudaEventRecord(e1, w->stream));
                CU(cudaEventSynchronize(e1));
                float ms = 0.0f;
                cudaEventElapsedTime(&ms, e0, e1);
                if (round == 1) tbest[mode] = ms;
            }
        if (!rc) rc = dbox_world_set_island_solver(w, tbest[1] < tbest[0] ? 1 : 0);
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (rc) return rc;
    if (choice) {
        if (cand[bi][0]) { choice[0] = 0; choice[1] = 0; choice[2] = 0; choice[3] = 1; choice[4] = cand[bi][1]; choice[5] = cand[bi][2]; }
        else { choice[0] = cand[bi][1]; choice[1] = cand[bi][2]; choice[2] = cand[bi][3]; choice[3] = 0; choice[4] = 0; choice[5] = 0; }
    }
    return rc;
}

int32_t dbox_world_set_phase_profile(dbox_world* w, int32_t enable) {
    if (!w) return DBOX_ERR_INVALID;
    w->profiling = enable ? 1 : 0;
    if (w->graph) { cudaGraphExecDestroy(w->graph); w->graph = nullptr; }
    if (w->tgraph) { cudaGraphExecDestroy(w->tgraph); w->tgraph = nullptr; }
    return DBOX_OK;
}

int32_t dbox_world_get_phase_profile(dbox_world* w, unsigned long long* out) {
    if (!w || !out) return DBOX_ERR_INVALID;
    if (!w->on_device || !w->d_prof.p) return DBOX_ERR_INVALID;
    CU(cudaStreamSynchronize(w->stream));
    CU(cudaMemcpy(out, w->d_prof.p, sizeof(unsigned long long) * dg::kProfSlots * w->worlds.size(), cudaMemcpyDeviceToHost));
    return DBOX_OK;
}

int32_t dbox_world_sync(dbox_world* w) {
    if (!w) return DBOX_ERR_INVALID;
    CU(cudaStreamSynchronize(w->stream));
    return DBOX_OK;
}

int32_t dbox_world_get_bodies(dbox_world* w, dbox_vec2* position, float* angle, dbox_vec2* linear_velocity,
                              float* angular_velocity, int32_t* awake) {
    if (!w) return DBOX_ERR_INVALID;
    std::vector<dbox_body_state> all;
    if (w->on_device && !w->dirty) {
        all.resize(w->total_bodies);
        CU(cudaStreamSynchronize(w->stream));
        if (w->total_bodies)
            CU(cudaMemcpy(all.data(), w->d_bs.p, sizeof(dbox_body_state) * all.size(), cudaMemcpyDeviceToHost));
    } else {
        for (auto& hw : w->worlds) all.insert(all.end(), hw.bs.begin(), hw.bs.end());
    }
    for (size_t i = 0; i < all.size(); ++i) {
        const dbox_body_state& b = all[i];
        if (position) { position[i].x = b.xf[0]; position[i].y = b.xf[1]; }
        if (angle) angle[i] = b.sweep[7];
        if (linear_velocity) { linear_velocity[i].x = b.vel[0]; linear_velocity[i].y = b.vel[1]; }
        if (angular_velocity) angular_velocity[i] = b.vel[2];
        if (awake) awake[i] = (b.flags & dg::kBodyAwake) ? 1 : 0;
    }
    return DBOX_OK;
}

int32_t dbox_world_body_count(dbox_world* w, int32_t world, int32_t* out) {
    if (!w || !out || world < 0 || world >= (int)w->worlds.size()) return DBOX_ERR_INVALID;
    *out = (int)w->worlds[world].bs.size();
    return DBOX_OK;
}

int32_t dbox_world_contact_count(dbox_world* w, int32_t world, int32_t* out) {
    if (!w || !out || world < 0 || world >= (int)w->worlds.size()) return DBOX_ERR_INVALID;
    if (w->on_device && !w->dirty) {
        dg::WorldDyn wd;
        CU(cudaStreamSynchronize(w->stream));
        CU(cudaMemcpy(&wd, w->d_wd.p + world, sizeof(wd), cudaMemcpyDeviceToHost));
        *out = wd.contact_count;
    } else {
        *out = (int)w->worlds[world].ct.size();
    }
    return DBOX_OK;
}

int32_t dbox_world_get_counts(dbox_world* w, int32_t world, int32_t* bodies, int32_t* joints, int32_t* contacts) {
    if (!w || world < 0 || world >= (int)w->worlds.size()) return fail(DBOX_ERR_INVALID, "dbox_world_get_counts: bad world");
    const HostWorld& hw = w->worlds[world];
    if (bodies) {
        int n = 0;
        for (int b = 0; b < (int)hw.bs.size(); ++b) n += body_gone(hw, b) ? 0 : 1;
        *bodies = n;
    }
    if (joints) {
        int n = 0;
        for (const dg::DJoint& j : hw.jt) n += j.type >= 0 ? 1 : 0;
        *joints = n;
    }
    if (contacts) return dbox_world_contact_count(w, world, contacts);
    return DBOX_OK;
}

int32_t dbox_world_export_state(dbox_world* w, int32_t world, dbox_world_header* header, dbox_body_state* bodies,
                                dbox_proxy_state* proxies, dbox_contact_state* contacts, dbox_joint_state* joints) {
    if (!w || world < 0 || world >= (int)w->worlds.size()) return fail(DBOX_ERR_INVALID, "export: bad world");
    if (w->on_device && !w->mirrors_fresh) {
        int rc = download(w);  // the device copy stays valid; only the mirrors refresh
        if (rc) return rc;
        if (!w->dirty && w->total_bodies + w->total_fixtures > 0) w->on_device = true;
    }
    const HostWorld& hw = w->worlds[world];
    if (header) {
        header->body_count = (int)hw.bs.size();
        header->fixture_count = (int)hw.fx.size();
        header->contact_count = (int)hw.ct.size();
        header->joint_count = (int)hw.jt.size();
        header->world_flags = (hw.wd.flags & ~4u) | (w->autoclear ? 4u : 0u);
        header->step_complete = hw.wd.step_complete;
        header->inv_dt0 = hw.wd.inv_dt0;
        header->reserved = 0;
    }
    if (bodies && !hw.bs.empty()) memcpy(bodies, hw.bs.data(), sizeof(dbox_body_state) * hw.bs.size());
    if (proxies && !hw.px.empty()) memcpy(proxies, hw.px.data(), sizeof(dbox_proxy_state) * hw.px.size());
    if (contacts) {
        for (size_t k = 0; k < hw.ct.size(); ++k) {
            dbox_contact_state c = hw.ct[k];
            for (int p = c.point_count; p < 2; ++p) memset(&c.points[p], 0, sizeof(c.points[p]));
            contacts[k] = c;
        }
    }
    if (joints) {
        for (size_t j = 0; j < hw.jt.size(); ++j) {
            joints[j].impulse[0] = hw.jt[j].impulse[0];
            joints[j].impulse[1] = hw.jt[j].impulse[1];
            joints[j].impulse[2] = hw.jt[j].impulse[2];
            joints[j].motor_impulse = hw.jt[j].motor_impulse;
            joints[j].limit_state = hw.jt[j].limit_state;
        }
    }
    return DBOX_OK;
}

int32_t dbox_world_import_state(dbox_world* w, int32_t world, const dbox_world_header* header,
                                const dbox_body_state* bodies, const dbox_proxy_state* proxies,
                                const dbox_contact_state* contacts, const dbox_joint_state* joints) {
    if (!w || !header || world < 0 || world >= (int)w->worlds.size()) return fail(DBOX_ERR_INVALID, "import: bad world");
    int rc = prepare_edit(w);
    if (rc) return rc;
    HostWorld& hw = w->worlds[world];
    if (header->body_count != (int)hw.bs.size() || header->fixture_count != (int)hw.fx.size() ||
        header->joint_count != (int)hw.jt.size())
        return fail(DBOX_ERR_INVALID, "import: world structure differs from the snapshot");
    if (header->body_count && !bodies) return fail(DBOX_ERR_INVALID, "import: bodies missing");
    if (header->fixture_count && !proxies) return fail(DBOX_ERR_INVALID, "import: proxies missing");
    if (header->contact_count && !contacts) return fail(DBOX_ERR_INVALID, "import: contacts missing");
    if (!hw.bs.empty()) memcpy(hw.bs.data(), bodies, sizeof(dbox_body_state) * hw.bs.size());
    if (!hw.px.empty()) memcpy(hw.px.data(), proxies, sizeof(dbox_proxy_state) * hw.px.size());
    hw.ct.assign(contacts, contacts + header->contact_count);
    for (auto& c : hw.ct) {
        if (c.fixture_a < 0 || c.fixture_a >= (int)hw.fx.size() || c.fixture_b < 0 || c.fixture_b >= (int)hw.fx.size())
            return fail(DBOX_ERR_INVALID, "import: contact fixture out of range");
    }
    if (joints) {
        for (size_t j = 0; j < hw.jt.size(); ++j) {
            hw.jt[j].impulse[0] = joints[j].impulse[0];
            hw.jt[j].impulse[1] = joints[j].impulse[1];
            hw.jt[j].impulse[2] = joints[j].impulse[2];
            hw.jt[j].motor_impulse = joints[j].motor_impulse;
            hw.jt[j].limit_state = joints[j].limit_state;
        }
    }
    hw.wd.flags = header->world_flags & ~2u;
    hw.wd.step_complete = header->step_complete;
    hw.wd.inv_dt0 = header->inv_dt0;
    hw.wd.contact_count = header->contact_count;
    return DBOX_OK;
}

// ---------------------------------------------------------------- world queries
// The device index of the fat AABBs (query.cu), rebuilt when device work ran since the last build.
static int query_prepare(dbox_world* w, dbox_query_buffers* b) {
    if (w->dirty || !w->on_device) {
        int rc = ensure_device(w);
        if (rc) return rc;
    }
    const int W = (int)w->worlds.size();
    const int nf = w->total_fixtures;
    int maxnf = 0;
    for (auto& hw : w->worlds) maxnf = std::max(maxnf, (int)hw.fx.size());
    const int words = std::max(1, (maxnf + 31) / 32);
    if (w->nsm <= 0) {
        int dev = 0;
        CU(cudaGetDevice(&dev));
        CU(cudaDeviceGetAttribute(&w->nsm, cudaDevAttrMultiProcessorCount, dev));
    }
    const int blocks = std::max(1, w->nsm * 8);
    if (w->q_box.n != (size_t)nf || w->q_live.n != (size_t)W) {
        if (w->q_box.alloc(nf) || w->q_idx.alloc(nf) || w->q_sidx0.alloc(nf) || w->q_sidx1.alloc(nf) ||
            w->q_key0.alloc(nf) || w->q_key1.alloc(nf) || w->q_bucket.alloc((size_t)nf / 32 + W + 2) ||
            w->q_group.alloc((size_t)nf / 1024 + W + 2) || w->q_live.alloc(W))
            return fail(DBOX_ERR_CUDA, "query index: out of device memory");
        w->q_gen = ~0ull;
    }
    if (w->q_bm_words < words || w->q_blocks != blocks) {
        const size_t n = (size_t)blocks * dbox_query_warps_per_block() * words;
        if (w->q_bitmap.alloc(n)) return fail(DBOX_ERR_CUDA, "query bitmaps: out of device memory");
        CU(cudaMemsetAsync(w->q_bitmap.p, 0, n * sizeof(unsigned), w->stream));
        w->q_bm_words = words;
        w->q_blocks = blocks;
    }
    b->W = W;
    b->wi = w->d_wi.p;
    b->fx = w->d_fx.p;
    b->px = w->d_px.p;
    b->bs = w->d_bs.p;
    b->box = w->q_box.p;
    b->idx = w->q_idx.p;
    b->bucket = w->q_bucket.p;
    b->group = w->q_group.p;
    b->live = w->q_live.p;
    b->key0 = w->q_key0.p;
    b->key1 = w->q_key1.p;
    b->sidx0 = w->q_sidx0.p;
    b->sidx1 = w->q_sidx1.p;
    b->bitmap = w->q_bitmap.p;
    b->bm_words = w->q_bm_words;
    b->query_blocks = w->q_blocks;
    if (w->q_gen != w->gen) {
        int err = dbox_launch_query_build(b, w->stream);
        if (err) return fail(DBOX_ERR_CUDA, "query index build: %s", cudaGetErrorString((cudaError_t)err));
        w->q_gen = w->gen;
    }
    return DBOX_OK;
}

int32_t dbox_world_query_aabb_device(dbox_world* w, int32_t n, const int32_t* world, const dbox_aabb* boxes,
                                     int32_t capacity, int32_t* counts, int32_t* fixtures) {
    if (!w || n < 0 || capacity < 0 || (n > 0 && (!world || !boxes || !counts || (capacity > 0 && !fixtures))))
        return fail(DBOX_ERR_INVALID, "dbox_world_query_aabb: bad arguments");
    dbox_query_buffers b;
    int rc = query_prepare(w, &b);
    if (rc) return rc;
    int err = dbox_launch_query_aabb(&b, n, world, boxes, capacity, counts, fixtures, w->stream);
    if (err) return fail(DBOX_ERR_CUDA, "query launch: %s", cudaGetErrorString((cudaError_t)err));
    return DBOX_OK;
}

int32_t dbox_world_raycast_device(dbox_world* w, int32_t n, const int32_t* world, const dbox_vec2* p1,
                                  const dbox_vec2* p2, int32_t mode, int32_t capacity, int32_t* counts,
                                  dbox_ray_hit* hits) {
    if (!w || n < 0 || (mode != DBOX_RAY_CLOSEST && mode != DBOX_RAY_ALL) || capacity < 0 ||
        (mode == DBOX_RAY_CLOSEST && capacity < 1) || (n > 0 && (!world || !p1 || !p2 || !counts || (capacity > 0 && !hits))))
        return fail(DBOX_ERR_INVALID, "dbox_world_raycast: bad arguments");
    dbox_query_buffers b;
    int rc = query_prepare(w, &b);
    if (rc) return rc;
    int err = dbox_launch_raycast(&b, n, world, p1, p2, mode, capacity, counts, hits, w->stream);
    if (err) return fail(DBOX_ERR_CUDA, "ray cast launch: %s", cudaGetErrorString((cudaError_t)err));
    return DBOX_OK;
}

// host-buffer forms: inputs packed into one upload, outputs read back in one copy each
static int query_stage(dbox_world* w, size_t in_bytes, size_t out_bytes) {
    if (w->q_in.n < in_bytes && w->q_in.alloc(in_bytes)) return fail(DBOX_ERR_CUDA, "query staging: out of device memory");
    if (w->q_out.n < out_bytes && w->q_out.alloc(out_bytes)) return fail(DBOX_ERR_CUDA, "query staging: out of device memory");
    return DBOX_OK;
}

static size_t align16(size_t v) { return (v + 15) & ~(size_t)15; }

int32_t dbox_world_query_aabb(dbox_world* w, int32_t n, const int32_t* world, const dbox_aabb* boxes,
                              int32_t capacity, int32_t* counts, int32_t* fixtures) {
    if (!w || n < 0 || capacity < 0 || (n > 0 && (!world || !boxes || !counts || (capacity > 0 && !fixtures))))
        return fail(DBOX_ERR_INVALID, "dbox_world_query_aabb: bad arguments");
    if (n == 0) return DBOX_OK;
    const size_t sw = align16(sizeof(int32_t) * n), sb = sizeof(dbox_aabb) * (size_t)n;
    const size_t sc = align16(sizeof(int32_t) * n), so = sizeof(int32_t) * (size_t)n * capacity;
    int rc = query_stage(w, sw + sb, sc + so);
    if (rc) return rc;
    unsigned char* in = w->q_in.p;
    unsigned char* out = w->q_out.p;
    CU(cudaMemcpyAsync(in, world, sizeof(int32_t) * n, cudaMemcpyHostToDevice, w->stream));
    CU(cudaMemcpyAsync(in + sw, boxes, sb, cudaMemcpyHostToDevice, w->stream));
    rc = dbox_world_query_aabb_device(w, n, (const int32_t*)in, (const dbox_aabb*)(in + sw), capacity, (int32_t*)out,
                                      (int32_t*)(out + sc));
    if (rc) return rc;
    CU(cudaMemcpyAsync(counts, out, sizeof(int32_t) * n, cudaMemcpyDeviceToHost, w->stream));
    if (so) CU(cudaMemcpyAsync(fixtures, out + sc, so, cudaMemcpyDeviceToHost, w->stream));
    CU(cudaStreamSynchronize(w->stream));
    return DBOX_OK;
}

int32_t dbox_world_raycast(dbox_world* w, int32_t n, const int32_t* world, const dbox_vec2* p1, const dbox_vec2* p2,
                           int32_t mode, int32_t capacity, int32_t* counts, dbox_ray_hit* hits) {
    if (!w || n < 0 || (mode != DBOX_RAY_CLOSEST && mode != DBOX_RAY_ALL) || capacity < 0 ||
        (mode == DBOX_RAY_CLOSEST && capacity < 1) || (n > 0 && (!world || !p1 || !p2 || !counts || (capacity > 0 && !hits))))
        return fail(DBOX_ERR_INVALID, "dbox_world_raycast: bad arguments");
    if (n == 0) return DBOX_OK;
    const size_t sw = align16(sizeof(int32_t) * n), sp = align16(sizeof(dbox_vec2) * (size_t)n);
    const size_t sc = align16(sizeof(int32_t) * n), so = sizeof(dbox_ray_hit) * (size_t)n * capacity;
    int rc = query_stage(w, sw + 2 * sp, sc + so);
    if (rc) return rc;
    unsigned char* in = w->q_in.p;
    unsigned char* out = w->q_out.p;
    CU(cudaMemcpyAsync(in, world, sizeof(int32_t) * n, cudaMemcpyHostToDevice, w->stream));
    CU(cudaMemcpyAsync(in + sw, p1, sizeof(dbox_vec2) * (size_t)n, cudaMemcpyHostToDevice, w->stream));
    CU(cudaMemcpyAsync(in + sw + sp, p2, sizeof(dbox_vec2) * (size_t)n, cudaMemcpyHostToDevice, w->stream));
    rc = dbox_world_raycast_device(w, n, (const int32_t*)in, (const dbox_vec2*)(in + sw), (const dbox_vec2*)(in + sw + sp),
                                   mode, capacity, (int32_t*)out, (dbox_ray_hit*)(out + sc));
    if (rc) return rc;
    CU(cudaMemcpyAsync(counts, out, sizeof(int32_t) * n, cudaMemcpyDeviceToHost, w->stream));
    if (so) CU(cudaMemcpyAsync(hits, out + sc, so, cudaMemcpyDeviceToHost, w->stream));
    CU(cudaStreamSynchronize(w->stream));
    return DBOX_OK;
}

// ---------------------------------------------------------------- b2World.Dump
// The text b2World.Dump logs (b2world.d:796-855, b2body.d:992-1022, b2fixture.d:280-358, the
// joints' Dump): statements that rebuild the world, floats as %.15e with an 'f' suffix.  The
// reference walks its body, fixture and joint lists, newest first: bodies[i] is body
// count - 1 - i, joints[k] joint count - 1 - k, and a body's fixtures come newest first.
namespace {
struct Dumper {
    std::string s;
    void put(const char* fmt, ...) __attribute__((format(printf, 2, 3))) {
        char tmp[512];
        va_list ap;
        va_start(ap, fmt);
        int n = vsnprintf(tmp, sizeof(tmp), fmt, ap);
        va_end(ap);
        s.append(tmp, n < (int)sizeof(tmp) ? n : (int)sizeof(tmp) - 1);
    }
    void vec(const char* in, const char* what, float x, float y) {
        put("%s%s.Set(%.15ef, %.15ef);\n", in, what, (double)x, (double)y);
    }
    void vec(const char* in, const char* what, float2 v) { vec(in, what, v.x, v.y); }
    void num(const char* in, const char* what, float v) { put("%s%s = %.15ef;\n", in, what, (double)v); }
    void flag(const char* in, const char* what, int v) { put("%s%s = bool(%d);\n", in, what, v); }

    void fixture(const HostWorld& hw, int fi, int body_index, const ChainRec* chain) {
        const dg::DFixture& f = hw.fx[fi];
        const char* in = "    ";
        put("    b2FixtureDef fd;\n");
        num(in, "fd.friction", f.friction);
        num(in, "fd.restitution", f.restitution);
        num(in, "fd.density", chain ? chain->density : f.density);
        put("    fd.isSensor = bool(%d);\n", f.sensor ? 1 : 0);
        put("    fd.filter.categoryBits = uint16(%d);\n", (int)(f.filter & 0xffffu));
        put("    fd.filter.maskBits = uint16(%d);\n", (int)(f.filter >> 16));
        put("    fd.filter.groupIndex = int16(%d);\n", f.group);
        if (chain) {
            const int n = (int)chain->v.size();
            put("    b2ChainShape shape;\n");
            put("    b2Vec2 vs[%d];\n", n);
            for (int i = 0; i < n; ++i) put("    vs[%d].Set(%.15ef, %.15ef);\n", i, (double)chain->v[i].x, (double)chain->v[i].y);
            put("    shape.CreateChain(vs, %d);\n", n);
            vec(in, "shape.m_prevVertex", chain->prev.x, chain->prev.y);
            vec(in, "shape.m_nextVertex", chain->next.x, chain->next.y);
            flag(in, "shape.m_hasPrevVertex", chain->has_prev ? 1 : 0);
            flag(in, "shape.m_hasNextVertex", chain->has_next ? 1 : 0);
        } else if (f.type == dg::kShapeCircle) {
            put("    b2CircleShape shape;\n");
            num(in, "shape.m_radius", f.radius);
            vec(in, "shape.m_p", f.v[0]);
        } else if (f.type == dg::kShapeEdge) {
            put("    b2EdgeShape shape;\n");
            num(in, "shape.m_radius", f.radius);
            vec(in, "shape.m_vertex0", f.v[2]);
            vec(in, "shape.m_vertex1", f.v[0]);
            vec(in, "shape.m_vertex2", f.v[1]);
            vec(in, "shape.m_vertex3", f.v[3]);
            flag(in, "shape.m_hasVertex0", f.edge_flags & 1);
            flag(in, "shape.m_hasVertex3", (f.edge_flags >> 1) & 1);
        } else {
            put("    b2PolygonShape shape;\n");
            put("    b2Vec2 vs[%d];\n", 8);                             // b2_maxPolygonVertices
            for (int i = 0; i < f.count; ++i) put("    vs[%d].Set(%.15ef, %.15ef);\n", i, (double)f.v[i].x, (double)f.v[i].y);
            put("    shape.Set(vs, %d);\n", f.count);
        }
        put("\n");
        put("    fd.shape = &shape;\n");
        put("\n");
        put("    bodies[%d].CreateFixture(&fd);\n", body_index);
    }

    void joint(const dg::DJoint& j, int index_a, int index_b, int index, const std::vector<int>& list_pos) {
        static const char* names[] = {"b2RevoluteJointDef", "b2DistanceJointDef", "b2RopeJointDef", "b2WeldJointDef",
                                      "b2FrictionJointDef", "b2MotorJointDef", "b2WheelJointDef", "b2PrismaticJointDef",
                                      "b2PulleyJointDef", "", "b2GearJointDef"};
        if (j.type == dg::kMouseJoint) {                                 // b2mousejoint.d:180-183
            put("Mouse joint dumping is not supported.\n");
            return;
        }
        const char* in = "  ";
        put("  %s jd;\n", names[j.type]);
        put("  jd.bodyA = bodies[%d];\n", index_a);
        put("  jd.bodyB = bodies[%d];\n", index_b);
        flag(in, "jd.collideConnected", j.collide_connected ? 1 : 0);
        const bool anchors = j.type != dg::kMotorJoint && j.type != dg::kPulleyJoint && j.type != dg::kGearJoint;
        if (j.type == dg::kPulleyJoint) {
            vec(in, "jd.groundAnchorA", j.ground_a);
            vec(in, "jd.groundAnchorB", j.ground_b);
        }
        if (anchors || j.type == dg::kPulleyJoint) {
            vec(in, "jd.localAnchorA", j.local_anchor_a);
            vec(in, "jd.localAnchorB", j.local_anchor_b);
        }
        switch (j.type) {
        case dg::kGearJoint:                                            // b2gearjoint.d:222-238
            put("  jd.joint1 = joints[%d];\n", list_pos[j.joint1]);
            put("  jd.joint2 = joints[%d];\n", list_pos[j.joint2]);
            num(in, "jd.ratio", j.ratio);
            break;
        case dg::kRevoluteJoint:                                        // b2revolutejoint.d:293-312
            num(in, "jd.referenceAngle", j.reference_angle);
            flag(in, "jd.enableLimit", j.enable_limit ? 1 : 0);
            num(in, "jd.lowerAngle", j.lower_angle);
            num(in, "jd.upperAngle", j.upper_angle);
            flag(in, "jd.enableMotor", j.enable_motor ? 1 : 0);
            num(in, "jd.motorSpeed", j.motor_speed);
            num(in, "jd.maxMotorTorque", j.max_motor_torque);
            break;
        case dg::kDistanceJoint:                                        // b2distancejoint.d:189-203
            num(in, "jd.length", j.length);
            num(in, "jd.frequencyHz", j.frequency_hz);
            num(in, "jd.dampingRatio", j.damping_ratio);
            break;
        case dg::kRopeJoint:                                            // b2ropejoint.d:145-157
            num(in, "jd.maxLength", j.length);
            break;
        case dg::kWeldJoint:                                            // b2weldjoint.d:174-188
            num(in, "jd.referenceAngle", j.reference_angle);
            num(in, "jd.frequencyHz", j.frequency_hz);
            num(in, "jd.dampingRatio", j.damping_ratio);
            break;
        case dg::kFrictionJoint:                                        // b2frictionjoint.d:157-170
            num(in, "jd.maxForce", j.max_force);
            num(in, "jd.maxTorque", j.max_torque);
            break;
        case dg::kMotorJoint:                                           // b2motorjoint.d:201-215
            vec(in, "jd.linearOffset", j.linear_offset);
            num(in, "jd.angularOffset", j.angular_offset);
            num(in, "jd.maxForce", j.max_force);
            num(in, "jd.maxTorque", j.max_torque);
            num(in, "jd.correctionFactor", j.correction_factor);
            break;
        case dg::kWheelJoint:                                           // b2wheeljoint.d:277-294
            vec(in, "jd.localAxisA", j.local_axis_x);
            flag(in, "jd.enableMotor", j.enable_motor ? 1 : 0);
            num(in, "jd.motorSpeed", j.motor_speed);
            num(in, "jd.maxMotorTorque", j.max_motor_torque);
            num(in, "jd.frequencyHz", j.frequency_hz);
            num(in, "jd.dampingRatio", j.damping_ratio);
            break;
        case dg::kPrismaticJoint:                                       // b2prismaticjoint.d:364-383
            vec(in, "jd.localAxisA", j.local_axis_x);
            num(in, "jd.referenceAngle", j.reference_angle);
            flag(in, "jd.enableLimit", j.enable_limit ? 1 : 0);
            num(in, "jd.lowerTranslation", j.lower_translation);
            num(in, "jd.upperTranslation", j.upper_translation);
            flag(in, "jd.enableMotor", j.enable_motor ? 1 : 0);
            num(in, "jd.motorSpeed", j.motor_speed);
            num(in, "jd.maxMotorForce", j.max_motor_force);
            break;
        case dg::kPulleyJoint:                                          // b2pulleyjoint.d:207-223
            num(in, "jd.lengthA", j.length_a);
            num(in, "jd.lengthB", j.length_b);
            num(in, "jd.ratio", j.ratio);
            break;
        }
        put("  joints[%d] = m_world.CreateJoint(&jd);\n", index);
    }

    void world(const HostWorld& hw, float2 g) {
        // the world lists, newest first, without destroyed bodies and joints
        std::vector<int> bodies, joints, list_index(hw.bs.size(), -1);
        for (int b = (int)hw.bs.size() - 1; b >= 0; --b)
            if (!body_gone(hw, b)) {
                list_index[b] = (int)bodies.size();
                bodies.push_back(b);
            }
        for (int j = (int)hw.jt.size() - 1; j >= 0; --j)
            if (hw.jt[j].type >= 0) joints.push_back(j);
        const int nb = (int)bodies.size(), nj = (int)joints.size();
        put("b2Vec2 g(%.15ef, %.15ef);\n", (double)g.x, (double)g.y);
        put("m_world.SetGravity(g);\n");
        put("b2Body** bodies = cast(b2Body**)b2Alloc(%d * (b2Body*).sizeof);\n", nb);
        put("b2Joint joints = cast(b2Joint)b2Alloc(%d * (b2Joint).sizeof);\n", nj);
        for (int i = 0; i < nb; ++i) {
            const int b = bodies[i];
            const dbox_body_state& s = hw.bs[b];
            const dg::BodyStatic& st = hw.bst[b];
            const char* in = "  ";
            put("{\n");
            put("  b2BodyDef bd;\n");
            put("  bd.type = b2BodyType(%d);\n", s.type);
            vec(in, "bd.position", s.xf[0], s.xf[1]);
            num(in, "bd.angle", s.sweep[7]);
            vec(in, "bd.linearVelocity", s.vel[0], s.vel[1]);
            num(in, "bd.angularVelocity", s.vel[2]);
            num(in, "bd.linearDamping", st.lin_damping);
            num(in, "bd.angularDamping", st.ang_damping);
            flag(in, "bd.allowSleep", (int)(s.flags & 0x4u));
            flag(in, "bd.awake", (int)(s.flags & 0x2u));
            flag(in, "bd.fixedRotation", (int)(s.flags & 0x10u));
            flag(in, "bd.bullet", (int)(s.flags & 0x8u));
            flag(in, "bd.active", (int)(s.flags & 0x20u));
            num(in, "bd.gravityScale", st.gravity_scale);
            put("  bodies[%d] = m_world.CreateBody(&bd);\n", i);
            put("\n");
            const ChainRec* last = nullptr;
            for (int fi : hw.body_fix[b]) {
                const ChainRec* chain = nullptr;
                for (const ChainRec& c : hw.chains)
                    if (!c.dead && fi >= c.first && fi < c.first + (int)c.v.size() - 1) chain = &c;
                if (chain && chain == last) continue;                   // one fixture per chain
                last = chain;
                put("  {\n");
                fixture(hw, fi, i, chain);
                put("  }\n");
            }
            put("}\n");
        }
        std::vector<int> list_pos(hw.jt.size(), -1);                   // b2Joint.m_index
        for (int k = 0; k < nj; ++k) list_pos[joints[k]] = k;
        for (int pass = 0; pass < 2; ++pass)                            // gear joints last
            for (int k = 0; k < nj; ++k) {
                const dg::DJoint& j = hw.jt[joints[k]];
                if ((j.type == dg::kGearJoint) != (pass == 1)) continue;
                put("{\n");
                joint(j, list_index[j.body_a], list_index[j.body_b], k, list_pos);
                put("}\n");
            }
        put("b2Free(joints);\n");
        put("b2Free(bodies);\n");
        put("joints = null;\n");
        put("bodies = null;\n");
    }
};
}  // namespace

int32_t dbox_world_dump(dbox_world* w, int32_t world, char* buf, int64_t capacity, int64_t* out_length) {
    if (!w || world < 0 || world >= (int)w->worlds.size() || capacity < 0 || (capacity > 0 && !buf))
        return fail(DBOX_ERR_INVALID, "dbox_world_dump: bad arguments");
    if (w->on_device && !w->mirrors_fresh) {
        int rc = download(w);
        if (rc) return rc;
        if (!w->dirty && w->total_bodies + w->total_fixtures > 0) w->on_device = true;
    }
    Dumper d;
    d.world(w->worlds[world], w->gravity);
    if (capacity > 0) {
        const size_t n = d.s.size() < (size_t)capacity - 1 ? d.s.size() : (size_t)capacity - 1;
        memcpy(buf, d.s.data(), n);
        buf[n] = 0;
    }
    if (out_length) *out_length = (int64_t)d.s.size();
    return DBOX_OK;
}

int32_t dbox_world_get_stream(dbox_world* w, void** out) {
    if (!w || !out) return fail(DBOX_ERR_INVALID, "dbox_world_get_stream: bad arguments");
    *out = (void*)w->stream;
    return DBOX_OK;
}

int32_t dbox_world_get_profile(dbox_world* w, dbox_profile* out) {
    if (!w || !out) return DBOX_ERR_INVALID;
    *out = w->profile;
    return DBOX_OK;
}

int32_t dbox_world_last_launches(dbox_world* w, int32_t* out) {
    if (!w || !out) return DBOX_ERR_INVALID;
    *out = w->last_launches;
    return DBOX_OK;
}

// Batched narrowphase (b2CollidePolygons / b2CollidePolygonAndCircle / b2CollideCircles,
// collision/b2collidepolygon.d:127-254, b2collidecircle.d:29-164) on the GPU.
int32_t dbox_collide_manifolds(int32_t n, const dbox_shape_def* shape_a, const float* xf_a,
                               const dbox_shape_def* shape_b, const float* xf_b, dbox_contact_state* out) {
    if (n < 0 || (n > 0 && (!shape_a || !xf_a || !shape_b || !xf_b || !out)))
        return fail(DBOX_ERR_INVALID, "dbox_collide_manifolds: bad arguments");
    if (n == 0) return DBOX_OK;
    std::vector<dg::DFixture> fa(n), fb(n);
    for (int i = 0; i < n; ++i) {
        if (!build_fixture(shape_a + i, &fa[i]) || !build_fixture(shape_b + i, &fb[i]))
            return fail(DBOX_ERR_INVALID, "dbox_collide_manifolds: pair %d has a degenerate shape", i);
        if (fa[i].type == dg::kShapeCircle && fb[i].type == dg::kShapePolygon)
            return fail(DBOX_ERR_INVALID, "dbox_collide_manifolds: pair %d: polygon must come first", i);
    }
    std::vector<dbox_contact_state> init(n);
    memset(init.data(), 0, sizeof(dbox_contact_state) * n);
    DBuf<dg::DFixture> dfa, dfb;
    DBuf<float4> dxa, dxb;
    DBuf<dbox_contact_state> dout;
    if (dfa.alloc(n) || dfb.alloc(n) || dxa.alloc(n) || dxb.alloc(n) || dout.alloc(n)) {
        dfa.free(); dfb.free(); dxa.free(); dxb.free(); dout.free();
        return fail(DBOX_ERR_CUDA, "dbox_collide_manifolds: allocation failed");
    }
    int rc = DBOX_OK;
    if (cudaMemcpy(dfa.p, fa.data(), sizeof(dg::DFixture) * n, cudaMemcpyHostToDevice) != cudaSuccess ||
        cudaMemcpy(dfb.p, fb.data(), sizeof(dg::DFixture) * n, cudaMemcpyHostToDevice) != cudaSuccess ||
        cudaMemcpy(dxa.p, xf_a, sizeof(float4) * n, cudaMemcpyHostToDevice) != cudaSuccess ||
        cudaMemcpy(dxb.p, xf_b, sizeof(float4) * n, cudaMemcpyHostToDevice) != cudaSuccess ||
        cudaMemcpy(dout.p, init.data(), sizeof(dbox_contact_state) * n, cudaMemcpyHostToDevice) != cudaSuccess ||
        dbox_launch_collide_pairs(n, dfa.p, dxa.p, dfb.p, dxb.p, dout.p, 0) != 0 ||
        cudaMemcpy(out, dout.p, sizeof(dbox_contact_state) * n, cudaMemcpyDeviceToHost) != cudaSuccess)
        rc = fail(DBOX_ERR_CUDA, "dbox_collide_manifolds: %s", cudaGetErrorString(cudaGetLastError()));
    dfa.free(); dfb.free(); dxa.free(); dxb.free(); dout.free();
    return rc;
}

// ---------------------------------------------------------------- allocation-free narrowphase
// For callers that must not allocate device memory: code running where a
// cudaMalloc would stall or be refused (inside a real-time frame loop that has
// a no-allocation rule, under a memory budget enforced by another allocator,
// or in a process whose device memory is owned by a host engine).  The device
// memory this entry point needs lives in one file-scope array that every GPU
// which loads the library holds until the process exits; calls allocate nothing.
namespace {

constexpr int kNoAllocMaxPairs = 4096;   // pairs per call
constexpr int kNoAllocChunk = 32;        // pairs converted per host staging chunk (stack)

struct NoAllocScratch {
    dg::DFixture fa[kNoAllocMaxPairs];
    dg::DFixture fb[kNoAllocMaxPairs];
    float4 xa[kNoAllocMaxPairs];
    float4 xb[kNoAllocMaxPairs];
    dbox_contact_state out[kNoAllocMaxPairs];
};

// 4096 * (2*176 + 2*16 + 96) bytes = 1,966,080 bytes of device memory per GPU.
static __device__ __align__(256) NoAllocScratch g_noalloc_scratch;

std::mutex g_noalloc_mutex;
NoAllocScratch* g_noalloc_ptr[64] = {nullptr};   // device address of the array, per device ordinal

// Set-up, once per device, with that device current: the host-side name of the
// array is only a stand-in, so its device address is fetched here.
int noalloc_scratch(NoAllocScratch** out) {
    int dev = -1;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess || dev < 0 || dev >= 64)
        return fail(DBOX_ERR_CUDA, "dbox_collide_manifolds_noalloc: no current device (%s)", cudaGetErrorString(e));
    std::lock_guard<std::mutex> lock(g_noalloc_mutex);
    if (!g_noalloc_ptr[dev]) {
        void* p = nullptr;
        e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess || !p)
            return fail(DBOX_ERR_CUDA, "dbox_collide_manifolds_noalloc: cudaGetSymbolAddress failed (%s)",
                        cudaGetErrorString(e));
        g_noalloc_ptr[dev] = (NoAllocScratch*)p;
    }
    *out = g_noalloc_ptr[dev];
    return DBOX_OK;
}

}  // namespace

extern "C" int32_t dbox_collide_manifolds_noalloc(int32_t n, const dbox_shape_def* shape_a, const float* xf_a,
                                                  const dbox_shape_def* shape_b, const float* xf_b,
                                                  dbox_contact_state* out) {
    if (n < 0 || (n > 0 && (!shape_a || !xf_a || !shape_b || !xf_b || !out)))
        return fail(DBOX_ERR_INVALID, "dbox_collide_manifolds_noalloc: bad arguments");
    if (n > kNoAllocMaxPairs)
        return fail(DBOX_ERR_CAPACITY, "dbox_collide_manifolds_noalloc: %d pairs requested, at most %d per call",
                    n, kNoAllocMaxPairs);
    if (n == 0) return DBOX_OK;
    NoAllocScratch* d = nullptr;
    int rc = noalloc_scratch(&d);
    if (rc) return rc;
    dg::DFixture ca[kNoAllocChunk], cb[kNoAllocChunk];
    for (int base = 0; base < n; base += kNoAllocChunk) {
        int m = n - base < kNoAllocChunk ? n - base : kNoAllocChunk;
        for (int i = 0; i < m; ++i) {
            if (!build_fixture(shape_a + base + i, &ca[i]) || !build_fixture(shape_b + base + i, &cb[i]))
                return fail(DBOX_ERR_INVALID, "dbox_collide_manifolds_noalloc: pair %d has a degenerate shape", base + i);
            if (ca[i].type == dg::kShapeCircle && cb[i].type == dg::kShapePolygon)
                return fail(DBOX_ERR_INVALID, "dbox_collide_manifolds_noalloc: pair %d: polygon must come first", base + i);
        }
        CU(cudaMemcpy(d->fa + base, ca, sizeof(dg::DFixture) * m, cudaMemcpyHostToDevice));
        CU(cudaMemcpy(d->fb + base, cb, sizeof(dg::DFixture) * m, cudaMemcpyHostToDevice));
    }
    CU(cudaMemcpy(d->xa, xf_a, sizeof(float4) * n, cudaMemcpyHostToDevice));
    CU(cudaMemcpy(d->xb, xf_b, sizeof(float4) * n, cudaMemcpyHostToDevice));
    // the array keeps the previous call's manifolds: start from zero as dbox_collide_manifolds does
    CU(cudaMemset(d->out, 0, sizeof(dbox_contact_state) * n));
    int err = dbox_launch_collide_pairs(n, d->fa, d->xa, d->fb, d->xb, d->out, 0);
    if (err) return fail(DBOX_ERR_CUDA, "dbox_collide_manifolds_noalloc: launch: %s", cudaGetErrorString((cudaError_t)err));
    CU(cudaMemcpy(out, d->out, sizeof(dbox_contact_state) * n, cudaMemcpyDeviceToHost));
    return DBOX_OK;
}

// per-world step diagnostics: islands and TOI events of the last step
int32_t dbox_world_step_stats(dbox_world* w, int32_t world, int32_t* islands, int32_t* toi_events) {
    if (!w || world < 0 || world >= (int)w->worlds.size()) return DBOX_ERR_INVALID;
    if (!w->on_device) { if (islands) *islands = 0; if (toi_events) *toi_events = 0; return DBOX_OK; }
    dg::WorldDyn wd;
    CU(cudaStreamSynchronize(w->stream));
    CU(cudaMemcpy(&wd, w->d_wd.p + world, sizeof(wd), cudaMemcpyDeviceToHost));
    if (islands) *islands = wd.islands;
    if (toi_events) *toi_events = wd.toi_events;
    return DBOX_OK;
}

}  // extern "C"
