// b2World.Step on the GPU: one team (a warp) per world for the ordered phases,
// flat grids for the per-contact narrowphase.
//
// Phase map (reference dbox src/dbox/dynamics/b2world.d:367-434):
//   k_step_begin      FindNewContacts when fixtures were added (b2world.d:372-376)
//   k_collide         b2ContactManager.Collide per contact (b2contactmanager.d:251-317)
//   k_collide_finish  contacts woken later in list order, wake flags, listener events,
//                     stable compaction
//   k_solve_toi       per world: b2World.Solve (solve_world: island search
//                     b2world.d:930-1095, b2Island.Solve b2island.d:75-280 for all islands
//                     at once in reference constraint order, SynchronizeFixtures,
//                     FindNewContacts), then b2World.SolveTOI (toi_world:
//                     b2world.d:1127-1452), inv_dt0 and ClearForces
//   k_step_fused      option (dbox_world_set_fused_step): the four phases above for each
//                     world on its warp, x.steps whole steps in one launch
// Large worlds (4,096+ fixtures) take kernels of their own: k_begin_big, k_collide_finish_big,
// k_solve_big, k_pairs_block and k_finish_big_block (AddPair, SolveTOI's setup passes) on
// thread-block clusters, k_toi_big (SolveTOI's event loop) on a 512-thread block.
//
// Gauss-Seidel order: inside an island every constraint reads the velocities
// (positions) its predecessors in island order wrote.  The kernels assign each
// constraint the level 1 + max(level of the last earlier constraint on either of
// its dynamic bodies) and run levels in sequence with the constraints of one
// level in parallel; constraints of one level share no dynamic body, so every
// constraint reads exactly the values it would read in sequential order.
// Static and kinematic bodies are never written by the solver (zero inverse
// mass), so they create no ordering edges.
#include <cuda_runtime.h>
#include <stdint.h>

#include "world.cuh"

namespace dg {

constexpr int kWarp = 32;
constexpr int kNoWake = 0x7fffffff;
constexpr unsigned long long kHashEmpty = 0xffffffffffffffffull;

DG int lane_id() { return threadIdx.x & 31; }
// phase stamp for the optional per-world profile (slots 0..11), lane 0 only
DG void stamp(const Ctx& x, int w, int slot) {
    if (x.prof && (threadIdx.x & 31) == 0) x.prof[kProfSlots * (size_t)w + slot] = clock64();
}
DG void tsync() { __syncwarp(); }

// ------------------------------------------------------------ contact pair hash (existence test of AddPair)
DG unsigned long long pair_key(int fa, int fb) {
    int lo = fa < fb ? fa : fb, hi = fa < fb ? fb : fa;
    return ((unsigned long long)(unsigned)lo << 32) | (unsigned)hi;
}
DG unsigned hash_slot(unsigned long long k, int cap) {
    k ^= k >> 33; k *= 0xff51afd7ed558ccdull; k ^= k >> 33; k *= 0xc4ceb9fe1a85ec53ull; k ^= k >> 33;
    return (unsigned)(k & (unsigned long long)(cap - 1));
}
DG void hash_insert(const Ctx& x, const WorldInfo& wi, unsigned long long key) {
    unsigned h = hash_slot(key, wi.hash_cap);
    for (int probe = 0; probe < wi.hash_cap; ++probe) {
        unsigned long long* slot = x.hash + wi.hash_start + ((h + probe) & (wi.hash_cap - 1));
        unsigned long long prev = atomicCAS(slot, kHashEmpty, key);
        if (prev == kHashEmpty || prev == key) return;
    }
}
DG bool hash_contains(const Ctx& x, const WorldInfo& wi, unsigned long long key) {
    unsigned h = hash_slot(key, wi.hash_cap);
    for (int probe = 0; probe < wi.hash_cap; ++probe) {
        unsigned long long v = x.hash[wi.hash_start + ((h + probe) & (wi.hash_cap - 1))];
        if (v == key) return true;
        if (v == kHashEmpty) return false;
    }
    return false;
}
// rebuild the table of world w from its live contacts
DG void hash_rebuild(const Ctx& x, int w) {
    const WorldInfo& wi = x.wi[w];
    int lane = lane_id();
    for (int i = lane; i < wi.hash_cap; i += kWarp) x.hash[wi.hash_start + i] = kHashEmpty;
    tsync();
    int n = x.wd[w].contact_count;
    for (int k = lane; k < n; k += kWarp) {
        const dbox_contact_state& c = x.ct[wi.contact_start + k];
        hash_insert(x, wi, pair_key(c.fixture_a, c.fixture_b));
    }
    tsync();
}

// ------------------------------------------------------------ filters
// b2Body.ShouldCollide (b2body.d:1149-1170): called as bodyB.ShouldCollide(bodyA)
DG bool body_should_collide(const Ctx& x, int self, int other) {
    if (x.bs[self].type != kDynamicBody && x.bs[other].type != kDynamicBody) return false;
    const BodyStatic& s = x.bst[self];
    for (int e = 0; e < s.jadj_count; ++e) {
        if (x.jadj_other[s.jadj_start + e] == other) {
            if (x.jt[x.jadj_joint[s.jadj_start + e]].collide_connected == 0) return false;
        }
    }
    return true;
}
// b2ContactFilter.ShouldCollide (b2worldcallbacks.d:52-64), or the world's table filter
// (b2World.SetContactFilter with a class table: bit b of row a lets classes a and b collide),
// alone or together with the default rule
DG bool filter_should_collide(const Ctx& x, int w, const DFixture& a, const DFixture& b) {
    bool def;
    if (a.group == b.group && a.group != 0) {
        def = a.group > 0;
    } else {
        uint32_t catA = a.filter & 0xffffu, maskA = a.filter >> 16;
        uint32_t catB = b.filter & 0xffffu, maskB = b.filter >> 16;
        def = (maskA & catB) != 0 && (catA & maskB) != 0;
    }
    const int mode = x.fmode ? x.fmode[w] : 0;
    if (mode == 0) return def;
    const bool tab = (x.ftab[64 * (size_t)w + (a.fclass & 63)] >> (b.fclass & 63)) & 1ull;
    return mode == 1 ? (tab && def) : tab;
}

// ------------------------------------------------------------ b2Contact.Update (contacts/b2contact.d:270-356)
// Returns true when the touching state changed (the caller wakes both bodies).
// `toi`: a sub-step update of SolveTOI, where a contact the host's PreSolve window disabled in
// this step stays disabled (the window's decision stands in for PreSolve's there).
DG bool contact_update(const Ctx& x, dbox_contact_state& c, unsigned* evt = nullptr, bool toi = false) {
    Manifold m;
    manifold_load(c, m);
    Manifold old = m;
    const bool userOff = toi && (c.flags & kContactUserOff) != 0;
    c.flags |= kContactEnabled;
    if (!toi) c.flags &= ~(uint32_t)kContactUserOff;
    bool wasTouching = (c.flags & kContactTouching) != 0;
    const DFixture& fa = x.fx[c.fixture_a];
    const DFixture& fb = x.fx[c.fixture_b];
    bool sensor = fa.sensor || fb.sensor;
    Xf xfA = b_xf(x.bs[fa.body]);
    Xf xfB = b_xf(x.bs[fb.body]);
    bool touching;
    bool changed = false;
    if (sensor) {
        touching = shapes_overlap(fa, xfA, fb, xfB);
        m.pointCount = 0;
    } else {
        evaluate_manifold(m, fa, xfA, fb, xfB);
        touching = m.pointCount > 0;
        unsigned fresh = 0;
        for (int i = 0; i < m.pointCount; ++i) {
            m.ni[i] = 0.0f;
            m.ti[i] = 0.0f;
            bool matched = false;
            for (int j = 0; j < old.pointCount; ++j) {
                if (old.id[j] == m.id[i]) { m.ni[i] = old.ni[j]; m.ti[i] = old.ti[j]; matched = true; break; }
            }
            if (!matched) fresh |= i == 0 ? (unsigned)kContactNew0 : (unsigned)kContactNew1;
        }
        if (x.ws_mode) c.flags = (c.flags & ~(uint32_t)(kContactNew0 | kContactNew1)) | fresh;
        changed = touching != wasTouching;
    }
    if (touching) c.flags |= kContactTouching; else c.flags &= ~(uint32_t)kContactTouching;
    if (userOff && !sensor && touching) c.flags &= ~(uint32_t)kContactEnabled;
    manifold_store(m, c);
    // listener calls of b2Contact.Update (b2contact.d:340-355): BeginContact, EndContact, PreSolve
    if (evt) *evt = (!wasTouching && touching ? 1u : 0u) | (wasTouching && !touching ? 2u : 0u) | (!sensor && touching ? 4u : 0u);
    return changed;
}

// ------------------------------------------------------------ contact-listener events
DG dbox_contact_event* world_events(const Ctx& x, const WorldInfo& wi, int w) {
    return x.events + 4 * (size_t)wi.contact_start + 64 * (size_t)w;
}
DG int world_event_cap(const WorldInfo& wi) { return 4 * wi.contact_cap + 64; }
DG void put_event(const Ctx& x, const WorldInfo& wi, int w, int slot, int kind, const dbox_contact_state& c,
                  int count, const float* ni, const float* ti) {
    if (slot >= world_event_cap(wi)) { set_error(x, w, DBOX_ERR_CAPACITY); return; }
    dbox_contact_event& e = world_events(x, wi, w)[slot];
    e.kind = kind;
    e.world = w;
    e.fixture_a = c.fixture_a - wi.fix_start;
    e.fixture_b = c.fixture_b - wi.fix_start;
    e.point_count = count;
    e.normal_impulses[0] = ni ? ni[0] : 0.0f;
    e.normal_impulses[1] = ni && count > 1 ? ni[1] : 0.0f;
    e.tangent_impulses[0] = ti ? ti[0] : 0.0f;
    e.tangent_impulses[1] = ti && count > 1 ? ti[1] : 0.0f;
}
// one lane appends the listener events of b2Contact.Update in their order
DG void put_update_events(const Ctx& x, const WorldInfo& wi, int w, WorldDyn& wd, unsigned evt, const dbox_contact_state& c) {
    if (evt & 1u) put_event(x, wi, w, wd.ev_count++, DBOX_EVENT_BEGIN, c, c.point_count, nullptr, nullptr);
    if (evt & 2u) put_event(x, wi, w, wd.ev_count++, DBOX_EVENT_END, c, c.point_count, nullptr, nullptr);
    if (evt & 4u) put_event(x, wi, w, wd.ev_count++, DBOX_EVENT_PRESOLVE, c, c.point_count, nullptr, nullptr);
}

// Collide treatment of one contact at list position lp: 0 = updated, 2 = destroyed.
// Wakes are recorded into s_woken (minimum list position) instead of the flags.
DG int collide_one(const Ctx& x, dbox_contact_state& c, int lp, bool use_atomic, unsigned* evt) {
    const DFixture& fa = x.fx[c.fixture_a];
    const DFixture& fb = x.fx[c.fixture_b];
    int A = fa.body, B = fb.body;
    AABB pa, pb;
    const dbox_proxy_state& qa = x.px[c.fixture_a];
    const dbox_proxy_state& qb = x.px[c.fixture_b];
    pa.lo = v2(qa.fat_aabb[0], qa.fat_aabb[1]); pa.hi = v2(qa.fat_aabb[2], qa.fat_aabb[3]);
    pb.lo = v2(qb.fat_aabb[0], qb.fat_aabb[1]); pb.hi = v2(qb.fat_aabb[2], qb.fat_aabb[3]);
    bool wake;
    int result;
    if (!aabb_overlap(pa, pb)) {
        // b2ContactManager.Destroy + b2Contact.Destroy (b2contactmanager.d:183-246, b2contact.d:402-422)
        wake = c.point_count > 0 && !fa.sensor && !fb.sensor;
        result = 2;
        *evt = (c.flags & kContactTouching) ? 2u : 0u;                 // EndContact on Destroy
    } else {
        wake = contact_update(x, c, evt);
        result = 0;
    }
    if (wake) {
        if (use_atomic) { atomicMin(&x.s_woken[A], lp); atomicMin(&x.s_woken[B], lp); }
        else {
            if (x.s_woken[A] > lp) x.s_woken[A] = lp;
            if (x.s_woken[B] > lp) x.s_woken[B] = lp;
        }
    }
    return result;
}

// ------------------------------------------------------------ broad-phase: FindNewContacts
// b2BroadPhase.UpdatePairs (b2broadphase.d:139-195) + b2ContactManager.AddPair (b2contactmanager.d:52-176).
// Pairs are produced directly in (idA, idB) order: for each proxy a in ascending
// id, its partners b > a with a or b in the move buffer; duplicates never arise.
DG AABB proxy_fat(const Ctx& x, int f) {
    const dbox_proxy_state& p = x.px[f];
    AABB a;
    a.lo = v2(p.fat_aabb[0], p.fat_aabb[1]);
    a.hi = v2(p.fat_aabb[2], p.fat_aabb[3]);
    return a;
}

// ---- grid candidates for worlds with many proxies.  UpdatePairs wants every pair (a < b)
// of overlapping fat AABBs with a or b moved (b2broadphase.d:139-195); for a world of
// thousands of proxies testing all pairs on one warp is quadratic.  Instead the ordinary
// proxies are radix-sorted by the grid cell of their lower corner (cells as large as the
// largest ordinary extent, row-major ids), so a proxy's candidates lie in the cells of the
// rows cy-1 .. cy of its corners, columns cx-1 .. cx: one key range per row.  Proxies much
// wider than the mean (e.g. container walls) are tested against everything.  Partners are
// then ordered by id, which gives the same pair list as the all-pairs search.
constexpr int kSapMinProxies = 1024;

struct Sap {
    const unsigned* key;   // sorted cell ids of the ordinary proxies
    const float4* box;     // their fat AABBs, then those of the wide proxies
    const int* idx;        // their world-local proxy index | moved << 31
    int n;                 // ordinary proxies
    const int* wide;       // wide proxies (extent over 4x the mean): index | moved << 31
    int nwide;
    const int* cstart;     // per cell (and one past the last): the first sorted proxy in it or after it
    float ox, oy, inv;     // grid origin and 1 / cell size
    int ncx, ncy;          // cells per row, rows
};

DG int sap_cell(float v, float o, float inv, int n) {
    int c = (int)floorf((v - o) * inv);
    return c < 0 ? 0 : (c >= n ? n - 1 : c);
}

// Sort the world's ordinary proxies by cell (one warp; stable LSD radix sort, 8 bits a pass).
DG Sap sap_build(const Ctx& x, int w, int* hist) {
    const WorldInfo& wi = x.wi[w];
    const int lane = lane_id();
    const int f0 = wi.fix_start, nf = wi.fix_count;
    const int* ord = wi.proxy_order ? x.proxy_order + f0 : nullptr;   // ranks in proxy-id order
    auto PX = [ord](int r) { return ord ? ord[r] : r; };
    float lo[2] = {3.4e38f, 3.4e38f}, hi[2] = {-3.4e38f, -3.4e38f}, sum = 0.0f;
    int cnt = 0;
    for (int i = lane; i < nf; i += kWarp) {
        const dbox_proxy_state& p = x.px[f0 + PX(i)];
        if (p.proxy_id < 0) continue;
        ++cnt;
        sum += bmax(p.fat_aabb[2] - p.fat_aabb[0], p.fat_aabb[3] - p.fat_aabb[1]);
    }
    for (int o = 16; o > 0; o >>= 1) {
        cnt += __shfl_xor_sync(0xffffffffu, cnt, o);
        sum += __shfl_xor_sync(0xffffffffu, sum, o);
    }
    const float cut = 4.0f * sum / (float)(cnt > 0 ? cnt : 1);
    auto is_wide = [&](const dbox_proxy_state& p) {
        return bmax(p.fat_aabb[2] - p.fat_aabb[0], p.fat_aabb[3] - p.fat_aabb[1]) > cut;
    };
    float ext = 0.0f;
    for (int i = lane; i < nf; i += kWarp) {
        const dbox_proxy_state& p = x.px[f0 + PX(i)];
        if (p.proxy_id < 0 || is_wide(p)) continue;
        ext = bmax(ext, bmax(p.fat_aabb[2] - p.fat_aabb[0], p.fat_aabb[3] - p.fat_aabb[1]));
        for (int a = 0; a < 2; ++a) { lo[a] = bmin(lo[a], p.fat_aabb[a]); hi[a] = bmax(hi[a], p.fat_aabb[a]); }
    }
    for (int o = 16; o > 0; o >>= 1) {
        ext = bmax(ext, __shfl_xor_sync(0xffffffffu, ext, o));
        for (int a = 0; a < 2; ++a) {
            lo[a] = bmin(lo[a], __shfl_xor_sync(0xffffffffu, lo[a], o));
            hi[a] = bmax(hi[a], __shfl_xor_sync(0xffffffffu, hi[a], o));
        }
    }
    Sap s;
    float cellsz = ext > 1e-6f ? ext * 1.001f : 1.0f;
    // at most 4 cells per proxy (+ 64), so the cell table fits its scratch (larger cells only
    // widen the candidate ranges)
    float span = bmax(hi[0] - lo[0], hi[1] - lo[1]);
    if (span / cellsz > 4000.0f) cellsz = span / 4000.0f;
    s.ox = lo[0];
    s.oy = lo[1];
    const float cap = 4.0f * (float)nf + 64.0f;
    for (int it = 0;; ++it) {
        s.inv = 1.0f / cellsz;
        s.ncx = (int)((hi[0] - lo[0]) * s.inv) + 2;
        s.ncy = (int)((hi[1] - lo[1]) * s.inv) + 2;
        if ((float)s.ncx * (float)s.ncy <= cap) break;
        cellsz = it < 32 ? cellsz * 1.05f * sqrtf((float)s.ncx * (float)s.ncy / cap) : 4.0f * span + 1.0f;
    }
    if (!(s.ncx >= 1 && s.ncy >= 1 && s.ncx <= 65536 && s.ncy <= 65536)) {   // non-finite bounds: one cell
        s.ncx = 1;
        s.ncy = 1;
        s.inv = 0.0f;
    }
    unsigned* k0 = x.s_sapk[0] + f0;
    unsigned* k1 = x.s_sapk[1] + f0;
    int* i0 = x.s_sapi[0] + f0;
    int* i1 = x.s_sapi[1] + f0;
    int nv = 0;
    for (int base = 0; base < nf; base += kWarp) {   // ordinary proxies, in id order
        int i = base + lane;
        bool v = i < nf && x.px[f0 + PX(i)].proxy_id >= 0 && !is_wide(x.px[f0 + PX(i)]);
        unsigned bal = __ballot_sync(0xffffffffu, v);
        if (v) {
            int r = nv + __popc(bal & ((1u << lane) - 1u));
            const dbox_proxy_state& p = x.px[f0 + PX(i)];
            int cx = sap_cell(p.fat_aabb[0], s.ox, s.inv, s.ncx), cy = sap_cell(p.fat_aabb[1], s.oy, s.inv, s.ncy);
            k0[r] = (unsigned)(cy * s.ncx + cx);
            i0[r] = i;
        }
        nv += __popc(bal);
    }
    tsync();
    for (int pass = 0; pass < 3; ++pass) {           // cell ids < 2^24
        const int shift = 8 * pass;
        const unsigned* kin = pass & 1 ? k1 : k0;
        const int* iin = pass & 1 ? i1 : i0;
        unsigned* kout = pass & 1 ? k0 : k1;
        int* iout = pass & 1 ? i0 : i1;
        for (int b = lane; b < 256; b += kWarp) hist[b] = 0;
        tsync();
        for (int i = lane; i < nv; i += kWarp) atomicAdd(&hist[(kin[i] >> shift) & 255u], 1);
        tsync();
        int run = 0;
        for (int base = 0; base < 256; base += kWarp) {
            int v = hist[base + lane];
            int incl = v;
            for (int o = 1; o < 32; o <<= 1) {
                int t = __shfl_up_sync(0xffffffffu, incl, o);
                if (lane >= o) incl += t;
            }
            hist[base + lane] = run + incl - v;
            run += __shfl_sync(0xffffffffu, incl, 31);
        }
        tsync();
        for (int base = 0; base < nv; base += kWarp) {    // stable scatter, 32 keys at a time
            int i = base + lane;
            unsigned k = i < nv ? kin[i] : 0u;
            int d = i < nv ? (int)((k >> shift) & 255u) : 256 + lane;
            unsigned peers = __match_any_sync(0xffffffffu, d);
            if (i < nv) {
                int pos = hist[d] + __popc(peers & ((1u << lane) - 1u));
                kout[pos] = k;
                iout[pos] = iin[i];
            }
            tsync();
            if (i < nv && (peers & ((1u << lane) - 1u)) == 0) hist[d] += __popc(peers);
            tsync();
        }
    }
    // three passes: the sorted data is in the second buffer
    for (int r = lane; r < nv; r += kWarp) {
        int i = i1[r];
        const dbox_proxy_state& p = x.px[f0 + PX(i)];
        x.s_sapbox[f0 + r] = make_float4(p.fat_aabb[0], p.fat_aabb[1], p.fat_aabb[2], p.fat_aabb[3]);
        if (p.moved) i1[r] = i | (int)0x80000000;
    }
    int nw = 0;
    for (int base = 0; base < nf; base += kWarp) {   // wide proxies after them, indices in the free buffer
        int i = base + lane;
        bool v = i < nf && x.px[f0 + PX(i)].proxy_id >= 0 && is_wide(x.px[f0 + PX(i)]);
        unsigned bal = __ballot_sync(0xffffffffu, v);
        if (v) {
            int r = nw + __popc(bal & ((1u << lane) - 1u));
            const dbox_proxy_state& p = x.px[f0 + PX(i)];
            x.s_sapbox[f0 + nv + r] = make_float4(p.fat_aabb[0], p.fat_aabb[1], p.fat_aabb[2], p.fat_aabb[3]);
            i0[r] = p.moved ? (i | (int)0x80000000) : i;
        }
        nw += __popc(bal);
    }
    // cell table: cstart[c] = the first sorted index whose cell is >= c (cstart[ncell] = nv)
    const int ncell = s.ncx * s.ncy;
    int* cstart = x.s_sapcell + 8 * f0 + 130 * w;
    for (int c = lane; c <= ncell; c += kWarp) cstart[c] = nv;
    tsync();
    for (int r = lane; r < nv; r += kWarp)
        if (r == 0 || k1[r] != k1[r - 1]) cstart[k1[r]] = r;
    tsync();
    int carry = nv;                                  // suffix minimum, 32 cells at a time from the end
    for (int base = (ncell / kWarp) * kWarp; base >= 0; base -= kWarp) {
        const int c = base + lane;
        int v = c <= ncell ? cstart[c] : nv;
        for (int o = 1; o < 32; o <<= 1) {
            const int t = __shfl_down_sync(0xffffffffu, v, o);
            if (lane + o < 32 && t < v) v = t;
        }
        if (carry < v) v = carry;
        if (c <= ncell) cstart[c] = v;
        carry = __shfl_sync(0xffffffffu, v, 0);
    }
    tsync();
    s.cstart = cstart;
    s.key = k1;
    s.box = x.s_sapbox + f0;
    s.idx = i1;
    s.n = nv;
    s.wide = i0;
    s.nwide = nw;
    return s;
}

// fn(b) for every partner b > a of proxy a (overlapping fat AABBs, a or b moved)
template <class F>
DG void sap_partners(const Sap& s, const AABB& fa, int a, bool amoved, F&& fn) {
    auto test = [&](int bi, const float4& bb) {
        int b = bi & 0x7fffffff;
        if (b <= a || (!amoved && bi >= 0)) return;
        AABB fb;
        fb.lo = v2(bb.x, bb.y);
        fb.hi = v2(bb.z, bb.w);
        if (aabb_overlap(fa, fb)) fn(b);
    };
    const int cx0 = sap_cell(fa.lo.x, s.ox, s.inv, s.ncx), cy0 = sap_cell(fa.lo.y, s.oy, s.inv, s.ncy);
    const int cx1 = sap_cell(fa.hi.x, s.ox, s.inv, s.ncx), cy1 = sap_cell(fa.hi.y, s.oy, s.inv, s.ncy);
    const int xa = cx0 > 0 ? cx0 - 1 : 0;
    for (int cy = cy0 > 0 ? cy0 - 1 : 0; cy <= cy1; ++cy) {
        const int klo = cy * s.ncx + xa, khi = cy * s.ncx + cx1;
        const int qe = s.cstart[khi + 1];
        for (int q = s.cstart[klo]; q < qe; ++q) test(s.idx[q], s.box[q]);
    }
    for (int q = 0; q < s.nwide; ++q) test(s.wide[q], s.box[s.n + q]);
}

// The pairs of UpdatePairs in (idA, idB) order into x.pairs (one warp); returns their count, or
// -1 when they overflow the world's pair buffer.  The move buffer is cleared.
template <bool kPerm>
__device__ __noinline__ int gen_pairs_warp_t(const Ctx& x, int w) {
    const WorldInfo& wi = x.wi[w];
    WorldDyn& wd = x.wd[w];
    int lane = lane_id();
    int f0 = wi.fix_start, nf = wi.fix_count;
    // proxies are walked by rank, in ascending proxy id (b2PairLessThan, b2broadphase.d:166):
    // the rank is the fixture index unless destruction let a newer fixture reuse a lower id
    const int* ord = x.proxy_order + f0;
    auto PX = [ord](int r) { return kPerm ? ord[r] : r; };          // the plain order needs no lookup
    // moved list, ascending rank
    int nm = 0;
    for (int base = 0; base < nf; base += kWarp) {
        int i = base + lane;
        bool mv = i < nf && x.px[f0 + PX(i)].moved && x.px[f0 + PX(i)].proxy_id >= 0;
        unsigned bal = __ballot_sync(0xffffffffu, mv);
        if (mv) x.s_moved[f0 + nm + __popc(bal & ((1u << lane) - 1))] = i;
        nm += __popc(bal);
    }
    tsync();
    if (nm == 0) return 0;
    __shared__ int sap_hist[kSolveWarps][256];
    const bool use_sap = nf >= kSapMinProxies;
    Sap sap;
    if (use_sap) sap = sap_build(x, w, sap_hist[(threadIdx.x >> 5) % kSolveWarps]);
    // count pairs per proxy a
    for (int a = lane; a < nf; a += kWarp) {
        int cnt = 0;
        if (use_sap) {
            if (x.px[f0 + PX(a)].proxy_id >= 0)
                sap_partners(sap, proxy_fat(x, f0 + PX(a)), a, x.px[f0 + PX(a)].moved != 0, [&](int) { ++cnt; });
        } else if (x.px[f0 + PX(a)].proxy_id >= 0) {
            AABB fa = proxy_fat(x, f0 + PX(a));
            if (x.px[f0 + PX(a)].moved) {
                for (int b = a + 1; b < nf; ++b)
                    if (x.px[f0 + PX(b)].proxy_id >= 0 && aabb_overlap(fa, proxy_fat(x, f0 + PX(b)))) ++cnt;
            } else {
                for (int m = 0; m < nm; ++m) {
                    int b = x.s_moved[f0 + m];
                    if (b > a && aabb_overlap(fa, proxy_fat(x, f0 + PX(b)))) ++cnt;
                }
            }
        }
        x.s_pcount[f0 + a] = cnt;
    }
    tsync();
    // exclusive scan of counts (warp, chunked)
    int total = 0;
    for (int base = 0; base < nf; base += kWarp) {
        int i = base + lane;
        int v = i < nf ? x.s_pcount[f0 + i] : 0;
        int incl = v;
        for (int o = 1; o < 32; o <<= 1) {
            int t = __shfl_up_sync(0xffffffffu, incl, o);
            if (lane >= o) incl += t;
        }
        if (i < nf) x.s_pcount[f0 + i] = total + incl - v;
        total += __shfl_sync(0xffffffffu, incl, 31);
    }
    tsync();
    if (total > wi.pair_cap) {
        if (lane == 0) set_error(x, w, DBOX_ERR_CAPACITY);
        return -1;
    }
    if (lane == 0) wd.acc_pairs += (unsigned long long)total;
    // fill pairs in (a, b) order
    for (int a = lane; a < nf; a += kWarp) {
        int o = x.s_pcount[f0 + a];
        if (x.px[f0 + PX(a)].proxy_id < 0) continue;
        AABB fa = proxy_fat(x, f0 + PX(a));
        if (use_sap) {
            int2* seg = x.pairs + wi.pair_start + o;
            int cnt = 0;
            sap_partners(sap, fa, a, x.px[f0 + PX(a)].moved != 0, [&](int b) { seg[cnt++] = make_int2(a, b); });
            for (int i = 1; i < cnt; ++i) {           // partners by id (insertion sort of ranks)
                int2 v = seg[i];
                int j = i - 1;
                while (j >= 0 && seg[j].y > v.y) { seg[j + 1] = seg[j]; --j; }
                seg[j + 1] = v;
            }
            for (int i = 0; i < cnt; ++i) seg[i] = make_int2(f0 + PX(seg[i].x), f0 + PX(seg[i].y));
        } else if (x.px[f0 + PX(a)].moved) {
            for (int b = a + 1; b < nf; ++b)
                if (x.px[f0 + PX(b)].proxy_id >= 0 && aabb_overlap(fa, proxy_fat(x, f0 + PX(b))))
                    x.pairs[wi.pair_start + o++] = make_int2(f0 + PX(a), f0 + PX(b));
        } else {
            for (int m = 0; m < nm; ++m) {
                int b = x.s_moved[f0 + m];
                if (b > a && aabb_overlap(fa, proxy_fat(x, f0 + PX(b))))
                    x.pairs[wi.pair_start + o++] = make_int2(f0 + PX(a), f0 + PX(b));
            }
        }
    }
    tsync();
    // clear the move buffer
    for (int i = lane; i < nf; i += kWarp) x.px[f0 + PX(i)].moved = 0;
    return total;
}

__device__ __forceinline__ int gen_pairs_warp(const Ctx& x, int w) {
    return x.wi[w].proxy_order ? gen_pairs_warp_t<true>(x, w) : gen_pairs_warp_t<false>(x, w);
}

// b2ContactManager.AddPair (b2contactmanager.d:52-176) for the world's `total` pairs in x.pairs,
// in pair order (one warp)
// exclusive prefix of v over the block in thread order; *total gets the sum (all threads)
DG int block_scan_value(int v, int* sh, int* total) {
    const int lane = lane_id(), warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    int incl = v;
    for (int o = 1; o < 32; o <<= 1) {
        const int t = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += t;
    }
    __syncthreads();
    if (lane == 31) sh[warp] = incl;
    __syncthreads();
    int before = 0, all = 0;
    for (int q = 0; q < nw; ++q) {
        before += q < warp ? sh[q] : 0;
        all += sh[q];
    }
    *total = all;
    return before + incl - v;
}

// The threads that run one world's SolveTOI together: a warp (every world with the rest of its
// step) or a block (a large world, after its pair search).  The lead (rank 0) does the serial
// parts of the event loop; the passes over the contact list are spread over the team, and
// the ones whose hits must be handled in list order hand them to the lead in that order.
struct WarpTeam {
    static constexpr bool kLists = false;        // joins and invalidations scan the candidate list
    DG int rank() const { return lane_id(); }
    DG int size() const { return kWarp; }
    DG bool lead() const { return lane_id() == 0; }
    DG void sync() const { __syncwarp(); }
    DG int bcast(int v) const { return __shfl_sync(0xffffffffu, v, 0); }
    // smallest (a, l) over the team: smallest a, then smallest l
    DG void argmin(float& a, int& l) const {
        for (int o = 16; o > 0; o >>= 1) {
            const float oa = __shfl_xor_sync(0xffffffffu, a, o);
            const int ol = __shfl_xor_sync(0xffffffffu, l, o);
            if (oa < a || (oa == a && ol < l)) { a = oa; l = ol; }
        }
    }
    // the lead calls f(t) for every t in [0, n) with pred(t), in descending t, until f returns
    // false; pred must not depend on what f changes
    template <class P, class F>
    DG void scan_desc(int n, P&& pred, F&& f, int lo = 0) const {
        const int lane = lane_id();
        bool stop = false;
        for (int base = n - 1; base >= lo && !stop; base -= kWarp) {
            const int t = base - lane;
            unsigned bal = __ballot_sync(0xffffffffu, t >= lo && pred(t));
            if (lane == 0) {
                while (bal) {
                    const int l = __ffs(bal) - 1;
                    bal &= bal - 1;
                    if (!f(base - l)) { stop = true; break; }
                }
            }
            __syncwarp();
            stop = __shfl_sync(0xffffffffu, stop, 0);
        }
    }
    // append every k in [k0, k1) with pred(k) to list[cnt ..] in ascending order; the new count
    template <class P>
    DG int collect(int k0, int k1, int* list, int cnt, P&& pred) const {
        const int lane = lane_id();
        for (int base = k0; base < k1; base += kWarp) {
            const int k = base + lane;
            const bool hit = k < k1 && pred(k);
            const unsigned bal = __ballot_sync(0xffffffffu, hit);
            if (hit) list[cnt + __popc(bal & ((1u << lane) - 1u))] = k;
            cnt += __popc(bal);
        }
        return cnt;
    }
    // f() is warp-collective and returns the same int on every lane
    template <class F>
    DG int first_warp(F&& f) const { return f(); }
    // exclusive prefix of a flag in rank order; *all gets the team's count
    DG int prefix(bool v, int* all) const {
        const unsigned bal = __ballot_sync(0xffffffffu, v);
        *all = __popc(bal);
        return __popc(bal & ((1u << lane_id()) - 1u));
    }
};

struct BlockTeam {
    static constexpr bool kLists = true;         // joins and invalidations walk per-body candidate lists
    unsigned* bal;                 // shared: one ballot per warp
    int* box;                      // shared: a broadcast slot
    float* ra;                     // shared: per-warp partial minima
    int* rl;
    unsigned* words;               // shared: one ballot per 32 positions of a scan (blockDim.x of them)
    int* aux;                      // shared: 4 counters of the incremental SolveTOI
    DG int rank() const { return threadIdx.x; }
    DG int size() const { return blockDim.x; }
    DG bool lead() const { return threadIdx.x == 0; }
    DG void sync() const { __syncthreads(); }
    DG int bcast(int v) const {
        __syncthreads();
        if (threadIdx.x == 0) box[0] = v;
        __syncthreads();
        return box[0];
    }
    DG void argmin(float& a, int& l) const {
        for (int o = 16; o > 0; o >>= 1) {
            const float oa = __shfl_xor_sync(0xffffffffu, a, o);
            const int ol = __shfl_xor_sync(0xffffffffu, l, o);
            if (oa < a || (oa == a && ol < l)) { a = oa; l = ol; }
        }
        __syncthreads();
        if (lane_id() == 0) { ra[threadIdx.x >> 5] = a; rl[threadIdx.x >> 5] = l; }
        __syncthreads();
        for (int k = 0; k < (int)(blockDim.x >> 5); ++k)
            if (ra[k] < a || (ra[k] == a && rl[k] < l)) { a = ra[k]; l = rl[k]; }
    }
    // positions [lo, n): 32 * blockDim.x at a time, every position's pred evaluated first (one
    // ballot word per 32 positions, each warp a share of the words, loads of consecutive words
    // in flight together), then a summary ballot per 32 words; the lead walks the non-empty
    // words in order
    template <class P, class F>
    DG void scan_desc(int n, P&& pred, F&& f, int lo = 0) const {
        const int nt = blockDim.x, nw = nt >> 5, warp = threadIdx.x >> 5, lane = lane_id();
        bool stop = false;
        for (int top = n - 1; top >= lo && !stop; top -= 32 * nt) {
            const int nq = (top - lo) / 32 + 1 < nt ? (top - lo) / 32 + 1 : nt;    // words in use
#pragma unroll 4
            for (int q = warp; q < nq; q += nw) {
                const int t = top - 32 * q - lane;
                const unsigned b = __ballot_sync(0xffffffffu, t >= lo && pred(t));
                if (lane == 0) words[q] = b;
            }
            __syncthreads();
            for (int g = warp; 32 * g < nq; g += nw) {
                const int q = 32 * g + lane;
                const unsigned any = __ballot_sync(0xffffffffu, q < nq && words[q] != 0u);
                if (lane == 0) bal[g] = any;
            }
            __syncthreads();
            if (threadIdx.x == 0) {
                for (int g = 0; 32 * g < nq && !stop; ++g) {
                    unsigned sm = bal[g];
                    while (sm && !stop) {
                        const int q = 32 * g + __ffs(sm) - 1;
                        sm &= sm - 1;
                        unsigned m = words[q];
                        while (m) {
                            const int l = __ffs(m) - 1;
                            m &= m - 1;
                            if (!f(top - 32 * q - l)) { stop = true; break; }
                        }
                    }
                }
                box[1] = stop;
            }
            __syncthreads();
            stop = box[1] != 0;
        }
        __syncthreads();
    }
    template <class P>
    DG int collect(int k0, int k1, int* list, int cnt, P&& pred) const {
        const int nt = blockDim.x, nw = nt >> 5, warp = threadIdx.x >> 5, lane = lane_id();
        for (int base = k0; base < k1; base += nt) {
            const int k = base + (int)threadIdx.x;
            const bool hit = k < k1 && pred(k);
            const unsigned b = __ballot_sync(0xffffffffu, hit);
            if (lane == 0) bal[warp] = b;
            __syncthreads();
            int before = 0, all = 0;
            for (int q = 0; q < nw; ++q) {
                const int c = __popc(bal[q]);
                before += q < warp ? c : 0;
                all += c;
            }
            if (hit) list[cnt + before + __popc(b & ((1u << lane) - 1u))] = k;
            cnt += all;
            __syncthreads();
        }
        return cnt;
    }
    template <class F>
    DG int first_warp(F&& f) const {
        int r = 0;
        if (threadIdx.x < kWarp) r = f();
        return bcast(r);
    }
    DG int prefix(bool v, int* all) const { return block_scan_value(v ? 1 : 0, rl, all); }
};

// b2ContactManager.AddPair's filters (b2contactmanager.d:52-120): same body, edge-edge (no such
// contact type), an existing contact, b2Body.ShouldCollide, the contact filter
DG bool pair_accept(const Ctx& x, int w, const WorldInfo& wi, int2 pr) {
    const DFixture& fA = x.fx[pr.x];
    const DFixture& fB = x.fx[pr.y];
    bool acc = fA.body != fB.body;
    if (acc) acc = !(fA.type == kShapeEdge && fB.type == kShapeEdge);
    if (acc) acc = !hash_contains(x, wi, pair_key(pr.x, pr.y));
    if (acc) acc = body_should_collide(x, fB.body, fA.body);
    if (acc) acc = filter_should_collide(x, w, fA, fB);
    return acc;
}
// b2Contact.Create and the rest of AddPair (b2contactmanager.d:120-176) into contact slot `slot`
DG void pair_create(const Ctx& x, const WorldInfo& wi, int2 pr, int slot) {
    // the registry's primary order puts the polygon before a circle and an edge before a circle
    // or a polygon (b2contact.d:358-400)
    int fa = pr.x, fb = pr.y;
    const int ta = x.fx[fa].type, tb = x.fx[fb].type;
    if ((ta == kShapeCircle && tb == kShapePolygon) || (ta != kShapeEdge && tb == kShapeEdge)) { int t = fa; fa = fb; fb = t; }
    const DFixture& FA = x.fx[fa];
    const DFixture& FB = x.fx[fb];
    dbox_contact_state& c = x.ct[wi.contact_start + slot];
    c.fixture_a = fa;
    c.fixture_b = fb;
    c.flags = kContactEnabled;
    c.toi_count = 0;
    c.toi = 0.0f;
    c.friction = fsqrt(FA.friction * FB.friction);                       // b2MixFriction
    c.restitution = FA.restitution > FB.restitution ? FA.restitution : FB.restitution;
    c.tangent_speed = 0.0f;
    c.point_count = 0;
    c.type = 0;
    c.local_normal[0] = c.local_normal[1] = 0.0f;
    c.local_point[0] = c.local_point[1] = 0.0f;
    for (int k = 0; k < 2; ++k) {
        c.points[k].local_point[0] = c.points[k].local_point[1] = 0.0f;
        c.points[k].normal_impulse = c.points[k].tangent_impulse = 0.0f;
        c.points[k].id = 0;
    }
    hash_insert(x, wi, pair_key(fa, fb));
    x.s_cbody[wi.contact_start + slot] = make_int2(FA.body - wi.body_start, FB.body - wi.body_start);
    x.s_cq[wi.contact_start + slot] = (unsigned char)((FA.sensor || FB.sensor) ? 2 : 0);
    if (!FA.sensor && !FB.sensor) {
        // SetAwake(true) on both bodies; concurrent writers store identical values
        dbox_body_state& ba = x.bs[FA.body];
        dbox_body_state& bb = x.bs[FB.body];
        if ((ba.flags & kBodyAwake) == 0) { atomicOr(&ba.flags, (unsigned)kBodyAwake); ba.sleep_time = 0.0f; }
        if ((bb.flags & kBodyAwake) == 0) { atomicOr(&bb.flags, (unsigned)kBodyAwake); bb.sleep_time = 0.0f; }
    }
}

// b2ContactManager.AddPair (b2contactmanager.d:52-176) for the pairs in order, new contacts
// appended in that order; a team of threads (a warp, or the block of a large world)
template <class Team>
__device__ __noinline__ void add_pairs_t(const Ctx& x, int w, int total, const Team& tm) {
    const WorldInfo& wi = x.wi[w];
    WorldDyn& wd = x.wd[w];
    const int rk = tm.rank(), ts = tm.size();
    int n = wd.contact_count;
    int added = 0;
    for (int base = 0; base < total; base += ts) {
        int i = base + rk;
        bool acc = false;
        int2 pr = make_int2(0, 0);
        if (i < total) {
            pr = x.pairs[wi.pair_start + i];
            acc = pair_accept(x, w, wi, pr);
        }
        int all;
        const int before = tm.prefix(acc, &all);
        if (acc) {
            int slot = n + added + before;
            if (slot < wi.contact_cap) pair_create(x, wi, pr, slot);
        }
        added += all;
        tm.sync();
    }
    if (n + added > wi.contact_cap) {
        if (tm.lead()) set_error(x, w, DBOX_ERR_CAPACITY);
        added = wi.contact_cap - n;
    }
    tm.sync();
    if (tm.lead()) wd.contact_count = n + added;
    tm.sync();
}

DG void add_pairs(const Ctx& x, int w, int total) { add_pairs_t(x, w, total, WarpTeam()); }

// b2ContactManager.FindNewContacts (b2contactmanager.d:320-323) on one warp
__device__ __noinline__ void find_new_contacts(const Ctx& x, int w) {
    const int total = gen_pairs_warp(x, w);
    if (total > 0) add_pairs(x, w, total);
}

// ------------------------------------------------------------ end-of-Solve pairs of a large world, one block
// The pairs gen_pairs_warp makes, in the same order, with a block's 1024 threads sharing the
// work: the ordinary proxies go into the same kind of grid (cell = lower corner, cells at
// least as large as any ordinary proxy) by a counting sort whose order inside a cell does not
// matter (each proxy's partners are sorted by rank), the wide ones into a list every proxy
// tests; partner counts, a block scan, then the fill.
// ---- thread-block clusters (a large world's block and its helpers)
DG unsigned cluster_rank() { unsigned r; asm volatile("mov.u32 %0, %%cluster_ctarank;" : "=r"(r)); return r; }
DG unsigned cluster_blocks() { unsigned r; asm volatile("mov.u32 %0, %%cluster_nctarank;" : "=r"(r)); return r; }
// every thread of every block of the cluster arrives (release) and waits (acquire): the
// global-memory writes made before it by any block are seen by the loads made after it
DG void cluster_sync() { asm volatile("barrier.cluster.arrive;\n\tbarrier.cluster.wait;" ::: "memory"); }
DG int ld_volatile_i(const int* p) { return *reinterpret_cast<const volatile int*>(p); }

constexpr int kPairThreads = 1024;

template <class T, class Op>
DG T block_reduce(T v, Op op, T* sh) {
    const int lane = lane_id(), warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
    for (int o = 16; o > 0; o >>= 1) v = op(v, __shfl_xor_sync(0xffffffffu, v, o));
    __syncthreads();
    if (lane == 0) sh[warp] = v;
    __syncthreads();
    v = sh[0];
    for (int k = 1; k < nwarps; ++k) v = op(v, sh[k]);
    return v;
}

// exclusive scan of a[0..n) in place; returns the total
DG int block_exclusive_scan(int* a, int n, int* sh) {
    const int lane = lane_id(), warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
    int carry = 0;
    for (int base = 0; base < n; base += blockDim.x) {
        const int i = base + (int)threadIdx.x;
        const int v = i < n ? a[i] : 0;
        int incl = v;
        for (int o = 1; o < 32; o <<= 1) {
            const int t = __shfl_up_sync(0xffffffffu, incl, o);
            if (lane >= o) incl += t;
        }
        __syncthreads();
        if (lane == 31) sh[warp] = incl;
        __syncthreads();
        if (warp == 0) {
            int sv = lane < nwarps ? sh[lane] : 0;
            for (int o = 1; o < 32; o <<= 1) {
                const int t = __shfl_up_sync(0xffffffffu, sv, o);
                if (lane >= o) sv += t;
            }
            if (lane < nwarps) sh[lane] = sv;
        }
        __syncthreads();
        const int before = warp > 0 ? sh[warp - 1] : 0;
        if (i < n) a[i] = carry + before + incl - v;
        carry += sh[nwarps - 1];
    }
    __syncthreads();
    return carry;
}

DG void sync_fixtures(const Ctx& x, int b);
// The same for a large world's end-of-step pairs on a cluster of csize blocks: each block takes
// chunks of blockDim.x pairs round-robin and counts the accepted ones (a rejected pair's first
// fixture gets its sign bit), the first block turns the chunk counts into offsets, then each
// chunk creates its accepted pairs at their places.  No pair occurs twice, so a pair's filters
// give the same answer whichever pairs were created before it.
DG void add_pairs_cluster(const Ctx& x, int w, int total, int csize, int crank, int* shi) {
    const WorldInfo& wi = x.wi[w];
    WorldDyn& wd = x.wd[w];
    const int tid = threadIdx.x, nt = blockDim.x;
    const int n = wd.contact_count;
    int2* pairs = x.pairs + wi.pair_start;
    int* chunk = x.s_pcount + wi.fix_start;                             // per chunk: count, then offset
    const int nch = (total + nt - 1) / nt;
    auto csync = [&]() { if (csize > 1) cluster_sync(); else __syncthreads(); };
    for (int c = crank; c < nch; c += csize) {
        const int i = c * nt + tid;
        bool acc = false;
        if (i < total) {
            const int2 pr = pairs[i];
            acc = pair_accept(x, w, wi, pr);
            if (!acc) pairs[i].x = pr.x | (int)0x80000000;
        }
        int all;
        block_scan_value(acc ? 1 : 0, shi, &all);
        if (tid == 0) chunk[c] = all;
    }
    if (crank == 0 && tid == 0) chunk[nch] = 0;
    csync();
    if (crank == 0) block_exclusive_scan(chunk, nch + 1, shi);
    csync();
    for (int c = crank; c < nch; c += csize) {
        const int i = c * nt + tid;
        int2 pr = make_int2(-1, 0);
        if (i < total) pr = pairs[i];
        const bool acc = i < total && pr.x >= 0;
        int all;
        const int before = block_scan_value(acc ? 1 : 0, shi, &all);
        const int slot = n + ld_volatile_i(&chunk[c]) + before;
        if (acc && slot < wi.contact_cap) pair_create(x, wi, pr, slot);
    }
    csync();
    if (crank == 0 && tid == 0) {
        int added = ld_volatile_i(&chunk[nch]);
        if (n + added > wi.contact_cap) {
            set_error(x, w, DBOX_ERR_CAPACITY);
            added = wi.contact_cap - n;
        }
        wd.contact_count = n + added;
    }
    __syncthreads();
}
// A large world's pair table and pair search on a block (pairs into x.pairs, their count into
// wd.pair_total).  At the end of Solve (b2world.d:1099-1120) after SynchronizeFixtures of the
// island bodies; at the start of a step (`at_begin`: FindNewContacts after fixtures were
// created, b2world.d:372-376) with the proxies as they stand.
DG void pairs_block(const Ctx& x, int w, bool at_begin, float* shf, int* shi, int csize, int crank) {
    const WorldInfo& wi = x.wi[w];
    WorldDyn& wd = x.wd[w];
    const int tid = threadIdx.x, nt = blockDim.x;
    // with a cluster (csize > 1) every block takes its round-robin share of the passes, the
    // first block the scans; block partials of the reductions are combined in block order
    const bool clustered = csize > 1, r0 = crank == 0;
    const int gtid = tid * csize + crank, gsize = nt * csize;
    auto csync = [&]() { if (clustered) cluster_sync(); else __syncthreads(); };
    const long long t_in = clock64();
    auto prof_out = [&]() { if (r0 && x.prof && tid == 0 && !at_begin) x.prof[kProfSlots * (size_t)w + 30] = clock64() - t_in; };
    if (!at_begin && (!(wd.step_complete && x.dt > 0.0f) || wd.error != 0)) {   // Solve did not reach its broad-phase
        if (r0 && tid == 0) { wd.pair_total = 0; wd.g_valid = 0; }
        prof_out();
        return;
    }
    // SynchronizeFixtures of the island bodies (b2world.d:1099-1116), the solve's last step
    if (!at_begin)
        for (int i = gtid; i < wi.body_count; i += gsize) {
            const int b = wi.body_start + i;
            if ((x.bs[b].flags & kBodyIsland) == 0 || x.bs[b].type == kStaticBody) continue;
            sync_fixtures(x, b);
        }
    // the contact pair table, rebuilt from the live contacts (hash_rebuild)
    for (int i = gtid; i < wi.hash_cap; i += gsize) x.hash[wi.hash_start + i] = kHashEmpty;
    csync();
    for (int k = gtid; k < wd.contact_count; k += gsize) {
        const dbox_contact_state& c = x.ct[wi.contact_start + k];
        hash_insert(x, wi, pair_key(c.fixture_a, c.fixture_b));
    }
    csync();
    const int f0 = wi.fix_start, nf = wi.fix_count;
    const int* ord = wi.proxy_order ? x.proxy_order + f0 : nullptr;
    auto PX = [ord](int r) { return ord ? ord[r] : r; };
    auto extent = [](const dbox_proxy_state& p) { return bmax(p.fat_aabb[2] - p.fat_aabb[0], p.fat_aabb[3] - p.fat_aabb[1]); };
    auto isum = [](int a, int b) { return a + b; };
    auto fsum = [](float a, float b) { return a + b; };
    auto fmn = [](float a, float b) { return bmin(a, b); };
    auto fmx = [](float a, float b) { return bmax(a, b); };
    // live proxies, moved ones, mean extent (the wide cut of sap_build)
    int cnt = 0, nm = 0;
    float sum = 0.0f;
    int* part = x.s_pcount + f0;                                         // 16 partials per block (cluster)
    for (int r = gtid; r < nf; r += gsize) {
        const dbox_proxy_state& p = x.px[f0 + PX(r)];
        if (p.proxy_id < 0) continue;
        ++cnt;
        sum += extent(p);
        if (p.moved) ++nm;
    }
    cnt = block_reduce(cnt, isum, shi);
    nm = block_reduce(nm, isum, shi);
    sum = block_reduce(sum, fsum, shf);
    if (clustered) {
        if (tid == 0) { part[16 * crank] = cnt; part[16 * crank + 1] = nm; part[16 * crank + 2] = __float_as_int(sum); }
        cluster_sync();
        cnt = 0; nm = 0; sum = 0.0f;
        for (int q = 0; q < csize; ++q) {
            cnt += ld_volatile_i(&part[16 * q]);
            nm += ld_volatile_i(&part[16 * q + 1]);
            sum += __int_as_float(ld_volatile_i(&part[16 * q + 2]));
        }
    }
    if (nm == 0 && !x.continuous) {                                     // no pairs, and no SolveTOI to serve
        if (r0 && tid == 0) { wd.pair_total = 0; wd.g_valid = 0; }
        prof_out();
        return;
    }
    const float cut = 4.0f * sum / (float)(cnt > 0 ? cnt : 1);
    float ext = 0.0f, lo0 = 3.4e38f, lo1 = 3.4e38f, hi0 = -3.4e38f, hi1 = -3.4e38f;
    int nv = 0;
    for (int r = gtid; r < nf; r += gsize) {
        const dbox_proxy_state& p = x.px[f0 + PX(r)];
        if (p.proxy_id < 0 || extent(p) > cut) continue;
        ++nv;
        ext = bmax(ext, extent(p));
        lo0 = bmin(lo0, p.fat_aabb[0]);
        lo1 = bmin(lo1, p.fat_aabb[1]);
        hi0 = bmax(hi0, p.fat_aabb[0]);
        hi1 = bmax(hi1, p.fat_aabb[1]);
    }
    nv = block_reduce(nv, isum, shi);
    ext = block_reduce(ext, fmx, shf);
    lo0 = block_reduce(lo0, fmn, shf);
    lo1 = block_reduce(lo1, fmn, shf);
    hi0 = block_reduce(hi0, fmx, shf);
    hi1 = block_reduce(hi1, fmx, shf);
    if (clustered) {
        if (tid == 0) {
            part[16 * crank + 3] = nv;
            part[16 * crank + 4] = __float_as_int(ext);
            part[16 * crank + 5] = __float_as_int(lo0);
            part[16 * crank + 6] = __float_as_int(lo1);
            part[16 * crank + 7] = __float_as_int(hi0);
            part[16 * crank + 8] = __float_as_int(hi1);
        }
        cluster_sync();
        nv = 0;
        for (int q = 0; q < csize; ++q) {
            nv += ld_volatile_i(&part[16 * q + 3]);
            ext = bmax(ext, __int_as_float(ld_volatile_i(&part[16 * q + 4])));
            lo0 = bmin(lo0, __int_as_float(ld_volatile_i(&part[16 * q + 5])));
            lo1 = bmin(lo1, __int_as_float(ld_volatile_i(&part[16 * q + 6])));
            hi0 = bmax(hi0, __int_as_float(ld_volatile_i(&part[16 * q + 7])));
            hi1 = bmax(hi1, __int_as_float(ld_volatile_i(&part[16 * q + 8])));
        }
    }
    // the grid (as sap_build sizes it)
    Sap s;
    float cellsz = ext > 1e-6f ? ext * 1.001f : 1.0f;
    const float span = bmax(hi0 - lo0, hi1 - lo1);
    if (span / cellsz > 4000.0f) cellsz = span / 4000.0f;
    s.ox = lo0;
    s.oy = lo1;
    const float capc = 4.0f * (float)nf + 64.0f;
    for (int it = 0;; ++it) {
        s.inv = 1.0f / cellsz;
        s.ncx = (int)((hi0 - lo0) * s.inv) + 2;
        s.ncy = (int)((hi1 - lo1) * s.inv) + 2;
        if ((float)s.ncx * (float)s.ncy <= capc) break;
        cellsz = it < 32 ? cellsz * 1.05f * sqrtf((float)s.ncx * (float)s.ncy / capc) : 4.0f * span + 1.0f;
    }
    if (!(s.ncx >= 1 && s.ncy >= 1 && s.ncx <= 65536 && s.ncy <= 65536)) {
        s.ncx = 1;
        s.ncy = 1;
        s.inv = 0.0f;
    }
    const int ncell = s.ncx * s.ncy;
    int* cstart = x.s_sapcell + 8 * f0 + 130 * w;                        // ncell + 1 entries
    int* cursor = cstart + 4 * nf + 65;                                  // ncell entries
    int* sidx = x.s_sapi[1] + f0;                                        // ordinary proxies by cell
    int* wide = x.s_sapi[0] + f0;                                        // wide proxies
    float4* box = x.s_sapbox + f0;                                       // their boxes, the wide ones after nv
    for (int c = gtid; c <= ncell; c += gsize) cstart[c] = 0;
    int* n_wide = &wd.g_nwide;                                           // counted here, then kept for SolveTOI
    if (r0 && tid == 0) *n_wide = 0;
    csync();
    for (int r = gtid; r < nf; r += gsize) {                             // counts per cell; the wide list
        const dbox_proxy_state& p = x.px[f0 + PX(r)];
        if (p.proxy_id < 0) continue;
        if (extent(p) > cut) {
            const int k = atomicAdd(n_wide, 1);
            wide[k] = p.moved ? (r | (int)0x80000000) : r;
            box[nv + k] = make_float4(p.fat_aabb[0], p.fat_aabb[1], p.fat_aabb[2], p.fat_aabb[3]);
        } else {
            const int cx = sap_cell(p.fat_aabb[0], s.ox, s.inv, s.ncx), cy = sap_cell(p.fat_aabb[1], s.oy, s.inv, s.ncy);
            atomicAdd(&cstart[cy * s.ncx + cx], 1);
        }
    }
    csync();
    if (r0) block_exclusive_scan(cstart, ncell + 1, shi);
    csync();
    for (int c = gtid; c < ncell; c += gsize) cursor[c] = cstart[c];
    csync();
    for (int r = gtid; r < nf; r += gsize) {                             // counting-sort scatter
        const dbox_proxy_state& p = x.px[f0 + PX(r)];
        if (p.proxy_id < 0 || extent(p) > cut) continue;
        const int cx = sap_cell(p.fat_aabb[0], s.ox, s.inv, s.ncx), cy = sap_cell(p.fat_aabb[1], s.oy, s.inv, s.ncy);
        const int slot = atomicAdd(&cursor[cy * s.ncx + cx], 1);
        sidx[slot] = p.moved ? (r | (int)0x80000000) : r;
        box[slot] = make_float4(p.fat_aabb[0], p.fat_aabb[1], p.fat_aabb[2], p.fat_aabb[3]);
    }
    csync();
    const int nwd = ld_volatile_i(n_wide);
    s.key = nullptr;
    s.box = box;
    s.idx = sidx;
    s.n = nv;
    s.wide = wide;
    s.nwide = nwd;
    s.cstart = cstart;
    if (r0 && tid == 0) {                                                // the grid, for SolveTOI's pair searches
        wd.g_ox = s.ox; wd.g_oy = s.oy; wd.g_inv = s.inv;
        wd.g_ncx = s.ncx; wd.g_ncy = s.ncy; wd.g_nv = nv; wd.g_valid = 1;
    }
    if (nm == 0) {
        if (r0 && tid == 0) wd.pair_total = 0;
        prof_out();
        return;
    }
    // partners per proxy.  An ordinary proxy finds its ordinary partners in the cells (a
    // pair is listed under its lower-ranked proxy, and needs one of the two moved); a wide
    // proxy finds its ordinary partners in the cells its box reaches (one thread per row of
    // cells) and its wide partners in the wide list, so no proxy tests the wide list.  Counts,
    // offsets, then the same passes fill the segments and each segment is sorted by partner.
    int* pcount = x.s_pcount + f0;
    int* pcur = x.s_moved + f0;
    // rows of cells per wide proxy, for the row jobs
    int* wrow = x.s_sapi[0] + f0 + nwd;                                  // nwd + 1 entries after the wide list
    for (int q = gtid; q <= nwd; q += gsize) {
        int rows = 0;
        if (q < nwd) {
            const float4 wb = box[nv + q];
            const int cy0 = sap_cell(wb.y, s.oy, s.inv, s.ncy), cy1 = sap_cell(wb.w, s.oy, s.inv, s.ncy);
            rows = cy1 - (cy0 > 0 ? cy0 - 1 : 0) + 1;
        }
        wrow[q] = rows;
    }
    csync();
    if (r0) block_exclusive_scan(wrow, nwd + 1, shi);
    csync();
    const int njobs = ld_volatile_i(&wrow[nwd]);
    auto wide_row = [&](int job, auto&& emit) {                          // job: one row of one wide proxy
        int q = 0, lo = 0, hi = nwd;                                     // the last q with wrow[q] <= job
        while (lo < hi) {
            const int mid = (lo + hi + 1) >> 1;
            if (wrow[mid] <= job) lo = mid; else hi = mid - 1;
        }
        q = lo;
        const int wi_ = wide[q];
        const int wr = wi_ & 0x7fffffff;
        const bool wmoved = wi_ < 0;
        const float4 wb = box[nv + q];
        AABB fw;
        fw.lo = v2(wb.x, wb.y);
        fw.hi = v2(wb.z, wb.w);
        const int cx0 = sap_cell(wb.x, s.ox, s.inv, s.ncx), cx1 = sap_cell(wb.z, s.ox, s.inv, s.ncx);
        const int cy0 = sap_cell(wb.y, s.oy, s.inv, s.ncy);
        const int cy = (cy0 > 0 ? cy0 - 1 : 0) + (job - wrow[q]);
        const int xa = cx0 > 0 ? cx0 - 1 : 0;
        const int qe = s.cstart[cy * s.ncx + cx1 + 1];
        for (int e = s.cstart[cy * s.ncx + xa]; e < qe; ++e) {
            const int bi = s.idx[e];
            if (!wmoved && bi >= 0) continue;
            const float4 bb = s.box[e];
            AABB fb;
            fb.lo = v2(bb.x, bb.y);
            fb.hi = v2(bb.z, bb.w);
            if (!aabb_overlap(fw, fb)) continue;
            const int b = bi & 0x7fffffff;
            emit(wr < b ? wr : b, wr < b ? b : wr);
        }
    };
    auto wide_wide = [&](int q, auto&& emit) {                           // wide q with wide v, ranks above q's
        const int wi_ = wide[q];
        const int wr = wi_ & 0x7fffffff;
        const float4 wb = box[nv + q];
        AABB fw;
        fw.lo = v2(wb.x, wb.y);
        fw.hi = v2(wb.z, wb.w);
        for (int v = 0; v < nwd; ++v) {
            const int vi = wide[v];
            const int vr = vi & 0x7fffffff;
            if (vr <= wr || (wi_ >= 0 && vi >= 0)) continue;
            const float4 vb = box[nv + v];
            AABB fv;
            fv.lo = v2(vb.x, vb.y);
            fv.hi = v2(vb.z, vb.w);
            if (aabb_overlap(fw, fv)) emit(wr, vr);
        }
    };
    Sap sc = s;                                                          // the cells alone
    sc.nwide = 0;
    for (int a = gtid; a < nf; a += gsize) {
        int c = 0;
        const dbox_proxy_state& p = x.px[f0 + PX(a)];
        if (p.proxy_id >= 0 && extent(p) <= cut)
            sap_partners(sc, proxy_fat(x, f0 + PX(a)), a, p.moved != 0, [&](int) { ++c; });
        pcount[a] = c;
    }
    csync();
    for (int job = gtid; job < njobs; job += gsize) wide_row(job, [&](int own, int) { atomicAdd(&pcount[own], 1); });
    for (int q = gtid; q < nwd; q += gsize) wide_wide(q, [&](int own, int) { atomicAdd(&pcount[own], 1); });
    csync();
    if (r0) {
        const int t = block_exclusive_scan(pcount, nf, shi);
        if (tid == 0) wd.pair_total = t;
    }
    csync();
    const int total = ld_volatile_i(&wd.pair_total);
    if (total > wi.pair_cap) {
        if (r0 && tid == 0) { set_error(x, w, DBOX_ERR_CAPACITY); wd.pair_total = 0; }
        prof_out();
        return;
    }
    int2* seg0 = x.pairs + wi.pair_start;
    for (int a = gtid; a < nf; a += gsize) {                             // ordinary partners first
        const dbox_proxy_state& p = x.px[f0 + PX(a)];
        int c = 0;
        if (p.proxy_id >= 0 && extent(p) <= cut) {
            int2* seg = seg0 + pcount[a];
            sap_partners(sc, proxy_fat(x, f0 + PX(a)), a, p.moved != 0, [&](int b) { seg[c++] = make_int2(a, b); });
        }
        pcur[a] = pcount[a] + c;
    }
    csync();
    auto put = [&](int own, int other) { seg0[atomicAdd(&pcur[own], 1)] = make_int2(own, other); };
    for (int job = gtid; job < njobs; job += gsize) wide_row(job, put);
    for (int q = gtid; q < nwd; q += gsize) wide_wide(q, put);
    csync();
    for (int a = gtid; a < nf; a += gsize) {                             // each segment by partner rank
        int2* seg = seg0 + pcount[a];
        const int d = (a + 1 < nf ? pcount[a + 1] : total) - pcount[a];
        int gap = 1;
        while (3 * gap + 1 < d) gap = 3 * gap + 1;
        for (; gap > 0; gap /= 3)
            for (int i = gap; i < d; ++i) {
                const int2 v = seg[i];
                int j = i - gap;
                while (j >= 0 && seg[j].y > v.y) { seg[j + gap] = seg[j]; j -= gap; }
                seg[j + gap] = v;
            }
        for (int i = 0; i < d; ++i) seg[i] = make_int2(f0 + PX(seg[i].x), f0 + PX(seg[i].y));
    }
    csync();
    for (int i = gtid; i < nf; i += gsize) x.px[f0 + i].moved = 0;      // the move buffer is consumed
    if (r0 && tid == 0) wd.acc_pairs += (unsigned long long)total;
    prof_out();
}

__global__ void __launch_bounds__(kPairThreads) k_pairs_block(const __grid_constant__ Ctx x) {
    __shared__ float shf[32];
    __shared__ int shi[32];
    const int csize = x.big_cluster > 1 ? (int)cluster_blocks() : 1;
    const int crank = csize > 1 ? (int)cluster_rank() : 0;
    pairs_block(x, x.big_worlds[blockIdx.x / csize], false, shf, shi, csize, crank);
}

// The start of a large world's step on its block: the wake marks of Collide cleared, and
// FindNewContacts when fixtures were just created (e_newFixture): the pair search, then AddPair
// (k_step_begin does both on a warp for the other worlds)
__global__ void __launch_bounds__(kPairThreads) k_begin_big(const __grid_constant__ Ctx x) {
    __shared__ float shf[32];
    __shared__ int shi[32];
    __shared__ unsigned s_bal[32];
    __shared__ int s_box[2];
    __shared__ float s_ra[32];
    __shared__ int s_rl[32];
    __shared__ int s_aux[4];
    const int w = x.big_worlds[blockIdx.x];
    const WorldInfo& wi = x.wi[w];
    for (int i = threadIdx.x; i < wi.body_count; i += blockDim.x) x.s_woken[wi.body_start + i] = kNoWake;
    if (!(x.wd[w].flags & 1u)) return;
    __syncthreads();
    pairs_block(x, w, true, shf, shi, 1, 0);
    __syncthreads();
    BlockTeam tm{s_bal, s_box, s_ra, s_rl, nullptr, s_aux};
    const int total = x.wd[w].pair_total;
    if (total > 0) add_pairs_t(x, w, total, tm);
    __syncthreads();
    if (threadIdx.x == 0) x.wd[w].flags &= ~1u;
}

// FindNewContacts inside SolveTOI for a large world (one warp): the move buffer holds the
// proxies this event's SynchronizeFixtures moved (ranks now[0 .. nnow)); their pairs with every
// overlapping proxy (b2BroadPhase.UpdatePairs, b2broadphase.d:139-195) come from the grid
// k_pairs_block left (its boxes are those after the solve) for proxies that have not moved
// since, and from a direct test against all[0 .. nall), the proxies moved during this SolveTOI
// (whose grid boxes are stale; toimv[rank] marks them).  Pairs are sorted into (idA, idB) order
// and left in the world's pair buffer; returns their count, or -1 when they overflow it.
DG int toi_pairs_big(const Ctx& x, int w, const int* now, int nnow, const int* all, int nall, const int* toimv) {
    const WorldInfo& wi = x.wi[w];
    const WorldDyn& wd = x.wd[w];
    const int lane = lane_id();
    const int f0 = wi.fix_start;
    const int* cstart = x.s_sapcell + 8 * f0 + 130 * w;
    const int* sidx = x.s_sapi[1] + f0;
    const int* wide = x.s_sapi[0] + f0;
    const float4* gbox = x.s_sapbox + f0;
    const float cs = wd.g_inv > 0.0f ? 1.0f / wd.g_inv : 0.0f;
    int2* out = x.pairs + wi.pair_start;
    int total = 0;
    auto emit = [&](bool hit, int ra, int rb) {                          // warp-collective append
        const unsigned bal = __ballot_sync(0xffffffffu, hit);
        if (hit) {
            const int slot = total + __popc(bal & ((1u << lane) - 1u));
            if (slot < wi.pair_cap) out[slot] = make_int2(ra < rb ? ra : rb, ra < rb ? rb : ra);
        }
        total += __popc(bal);
    };
    for (int q = 0; q < nnow; ++q) {
        const int ra = now[q];
        const AABB fa = proxy_fat(x, f0 + ra);
        // ordinary proxies by cell: lower corners within [lo - cell, hi] in both axes
        const int cx0 = sap_cell(fa.lo.x - cs, wd.g_ox, wd.g_inv, wd.g_ncx), cx1 = sap_cell(fa.hi.x, wd.g_ox, wd.g_inv, wd.g_ncx);
        const int cy0 = sap_cell(fa.lo.y - cs, wd.g_oy, wd.g_inv, wd.g_ncy), cy1 = sap_cell(fa.hi.y, wd.g_oy, wd.g_inv, wd.g_ncy);
        for (int cy = cy0; cy <= cy1; ++cy) {
            const int e0 = cstart[cy * wd.g_ncx + cx0], e1 = cstart[cy * wd.g_ncx + cx1 + 1];
            for (int base = e0; base < e1; base += kWarp) {
                const int e = base + lane;
                bool hit = false;
                int rb = 0;
                if (e < e1) {
                    rb = sidx[e] & 0x7fffffff;
                    if (rb != ra && !toimv[rb]) {
                        const float4 b = gbox[e];
                        AABB bb;
                        bb.lo = v2(b.x, b.y);
                        bb.hi = v2(b.z, b.w);
                        hit = aabb_overlap(fa, bb);
                    }
                }
                emit(hit, ra, rb);
            }
        }
        for (int base = 0; base < wd.g_nwide; base += kWarp) {            // wide proxies
            const int e = base + lane;
            bool hit = false;
            int rb = 0;
            if (e < wd.g_nwide) {
                rb = wide[e] & 0x7fffffff;
                if (rb != ra && !toimv[rb] && x.px[f0 + rb].proxy_id >= 0) hit = aabb_overlap(fa, proxy_fat(x, f0 + rb));
            }
            emit(hit, ra, rb);
        }
        for (int base = 0; base < nall; base += kWarp) {                  // proxies moved during SolveTOI
            const int e = base + lane;
            bool hit = false;
            int rb = 0;
            if (e < nall) {
                rb = all[e];
                // a pair of two proxies moved by this event is found from the lower one only
                bool both_now = false;
                for (int k = 0; k < nnow; ++k) both_now |= now[k] == rb;
                if (rb != ra && (!both_now || ra < rb)) hit = aabb_overlap(fa, proxy_fat(x, f0 + rb));
            }
            emit(hit, ra, rb);
        }
    }
    tsync();
    if (total > wi.pair_cap) {
        if (lane == 0) set_error(x, w, DBOX_ERR_CAPACITY);
        return -1;
    }
    if (lane == 0) {                                                     // (idA, idB) order
        for (int i = 1; i < total; ++i) {
            const int2 v = out[i];
            int j = i - 1;
            while (j >= 0 && (out[j].x > v.x || (out[j].x == v.x && out[j].y > v.y))) { out[j + 1] = out[j]; --j; }
            out[j + 1] = v;
        }
    }
    tsync();
    for (int i = lane; i < total; i += kWarp) out[i] = make_int2(f0 + out[i].x, f0 + out[i].y);
    for (int k = lane; k < nnow; k += kWarp) x.px[f0 + now[k]].moved = 0;          // the move buffer is consumed
    tsync();
    return total;
}

DG void toi_world(const Ctx& x, int w, float* sbp);

// ------------------------------------------------------------ kernels
// the start of b2World.Step (b2world.d:367-376) for world w on one warp: per-step records
// reset, wake marks cleared, FindNewContacts after fixtures were created
DG void step_begin_world(const Ctx& x, int w) {
    WorldDyn& wd = x.wd[w];
    const WorldInfo& wi = x.wi[w];
    int lane = lane_id();
    if (lane == 0) { wd.error = 0; wd.islands = 0; wd.toi_events = 0; wd.ev_count = 0; }
    if (!wi.pair_block)                                                 // large worlds: k_begin_big
        for (int i = lane; i < wi.body_count; i += kWarp) x.s_woken[wi.body_start + i] = kNoWake;
    tsync();
    if ((wd.flags & 1u) && !wi.pair_block) {                            // e_newFixture (large worlds: k_begin_big)
        hash_rebuild(x, w);
        find_new_contacts(x, w);
        if (lane == 0) wd.flags &= ~1u;
    }
}

__global__ void k_step_begin(const __grid_constant__ Ctx x) {
    int w = (blockIdx.x * blockDim.x + threadIdx.x) / kWarp;
    if (w >= x.W) return;
    step_begin_world(x, w);
}

// b2ContactManager.Collide (b2contactmanager.d:251-317) for contact slot i of world w: the
// contact filter, the active test and the narrow phase; the contacts of a world are
// independent here (wakes are only marked, in s_woken, and applied by the finish)
DG void collide_contact(const Ctx& x, int w, int i) {
    const WorldInfo& wi = x.wi[w];
    int k = i - wi.contact_start;
    int n = x.wd[w].contact_count;
    if (k >= n) return;
    int lp = n - 1 - k;
    dbox_contact_state c = x.ct[i];
    const DFixture& fa = x.fx[c.fixture_a];
    const DFixture& fb = x.fx[c.fixture_b];
    int A = fa.body, B = fb.body;
    int state = 0;
    unsigned evt = 0;
    if (c.flags & kContactFilter) {                                // b2contactmanager.d:266-288
        if (!body_should_collide(x, B, A) || !filter_should_collide(x, w, fa, fb)) {
            state = 2;
            evt = (c.flags & kContactTouching) ? 2u : 0u;
            if (c.point_count > 0 && !fa.sensor && !fb.sensor) {
                atomicMin(&x.s_woken[A], lp);
                atomicMin(&x.s_woken[B], lp);
            }
        } else {
            c.flags &= ~(uint32_t)kContactFilter;
        }
    }
    if (state == 0) {
        const dbox_body_state& ba = x.bs[A];
        const dbox_body_state& bb = x.bs[B];
        bool activeA = (ba.flags & kBodyAwake) && ba.type != kStaticBody;
        bool activeB = (bb.flags & kBodyAwake) && bb.type != kStaticBody;
        if (!activeA && !activeB) state = 1;
        else state = collide_one(x, c, lp, true, &evt);
    }
    x.s_cstate[i] = state;
    if (x.record_events) x.s_cevt[i] = (unsigned char)evt;
    if (state != 2) x.ct[i] = c;
}

__global__ void k_collide(Ctx x) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < x.total_contacts; i += gridDim.x * blockDim.x)
        collide_contact(x, x.c_world[i], i);
}

// Contacts skipped as inactive may become active when an earlier contact in list
// order woke one of their bodies (Collide walks the list and wakes as it goes).
// the end of b2ContactManager.Collide for world w on one warp: contacts revived by a wake,
// listener events, wakes, compaction
DG void collide_finish_world(const Ctx& x, int w) {
    const WorldInfo& wi = x.wi[w];
    WorldDyn& wd = x.wd[w];
    int lane = lane_id();
    int n = wd.contact_count;
    int c0 = wi.contact_start;
    // any inactive contact with a body woken during this Collide?
    bool need = false;
    for (int k = lane; k < n; k += kWarp) {
        if (x.s_cstate[c0 + k] == 1) {
            const dbox_contact_state& c = x.ct[c0 + k];
            int A = x.fx[c.fixture_a].body, B = x.fx[c.fixture_b].body;
            if (x.s_woken[A] != kNoWake || x.s_woken[B] != kNoWake) need = true;
        }
    }
    need = __any_sync(0xffffffffu, need);
    if (need && lane == 0) {
        for (int k = n - 1; k >= 0; --k) {
            if (x.s_cstate[c0 + k] != 1) continue;
            int lp = n - 1 - k;
            dbox_contact_state& c = x.ct[c0 + k];
            int A = x.fx[c.fixture_a].body, B = x.fx[c.fixture_b].body;
            const dbox_body_state& ba = x.bs[A];
            const dbox_body_state& bb = x.bs[B];
            bool awA = (ba.flags & kBodyAwake) || x.s_woken[A] < lp;
            bool awB = (bb.flags & kBodyAwake) || x.s_woken[B] < lp;
            bool activeA = awA && ba.type != kStaticBody;
            bool activeB = awB && bb.type != kStaticBody;
            if (!activeA && !activeB) continue;
            unsigned evt = 0;
            x.s_cstate[c0 + k] = collide_one(x, c, lp, false, &evt);
            if (x.record_events) x.s_cevt[c0 + k] = (unsigned char)evt;
        }
    }
    tsync();
    // listener events of this Collide, in list order (newest contact first)
    if (x.record_events) {
        int base = 0;
        for (int top = n - 1; top >= 0; top -= kWarp) {
            int k = top - lane;
            unsigned evt = k >= 0 ? x.s_cevt[c0 + k] : 0u;
            int cnt = __popc(evt);
            int incl = cnt;
            for (int o = 1; o < 32; o <<= 1) {
                int t = __shfl_up_sync(0xffffffffu, incl, o);
                if (lane >= o) incl += t;
            }
            if (cnt) {
                const dbox_contact_state& c = x.ct[c0 + k];
                int slot = base + incl - cnt;
                if (evt & 1u) put_event(x, wi, w, slot++, DBOX_EVENT_BEGIN, c, c.point_count, nullptr, nullptr);
                if (evt & 2u) put_event(x, wi, w, slot++, DBOX_EVENT_END, c, c.point_count, nullptr, nullptr);
                if (evt & 4u) put_event(x, wi, w, slot++, DBOX_EVENT_PRESOLVE, c, c.point_count, nullptr, nullptr);
            }
            base += __shfl_sync(0xffffffffu, incl, 31);
        }
        if (lane == 0) wd.ev_count = base;
        tsync();
    }
    // apply wakes
    for (int i = lane; i < wi.body_count; i += kWarp) {
        int b = wi.body_start + i;
        if (x.s_woken[b] != kNoWake) b_set_awake(x.bs[b], true);
    }
    // stable compaction of surviving contacts
    int out = 0;
    for (int base = 0; base < n; base += kWarp) {
        int k = base + lane;
        bool keep = k < n && x.s_cstate[c0 + k] != 2;
        dbox_contact_state c;
        if (keep) c = x.ct[c0 + k];
        unsigned bal = __ballot_sync(0xffffffffu, keep);
        tsync();
        if (keep) x.ct[c0 + out + __popc(bal & ((1u << lane) - 1))] = c;
        out += __popc(bal);
        tsync();
    }
    if (lane == 0) { wd.contact_count = out; wd.acc_contacts += (unsigned long long)n; wd.acc_steps += 1; }
    tsync();
}

__global__ void k_collide_finish(Ctx x) {
    int w = (blockIdx.x * blockDim.x + threadIdx.x) / kWarp;
    if (w >= x.W) return;
    if (x.wi[w].pair_block) return;                                     // k_collide_finish_big
    collide_finish_world(x, w);
}

// the Collide part of one step of world w on one warp (k_step_fused): the step's start, every
// contact's narrow phase over the lanes, the finish
__device__ __noinline__ void collide_world(const Ctx& x, int w) {
    step_begin_world(x, w);
    tsync();
    const int c0 = x.wi[w].contact_start, n = x.wd[w].contact_count;
    for (int k = lane_id(); k < n; k += kWarp) collide_contact(x, w, c0 + k);
    tsync();
    collide_finish_world(x, w);
}

// ------------------------------------------------------------ solver body state
// b2Position / b2Velocity of the island solver (dynamics/b2timestep.d:61-72) for every
// body of a world, by world-local body index: vx vy w cx cy a.  Shared memory when the
// world fits, else a global scratch row.
struct SB {
    float* p;
    DG float2 v(int i) const { return v2(p[6 * i], p[6 * i + 1]); }
    DG float w(int i) const { return p[6 * i + 2]; }
    DG float2 c(int i) const { return v2(p[6 * i + 3], p[6 * i + 4]); }
    DG float a(int i) const { return p[6 * i + 5]; }
    DG void set_v(int i, float2 v, float w) { p[6 * i] = v.x; p[6 * i + 1] = v.y; p[6 * i + 2] = w; }
    DG void set_c(int i, float2 c, float a) { p[6 * i + 3] = c.x; p[6 * i + 4] = c.y; p[6 * i + 5] = a; }
};

DG void sb_load(SB sb, int i, const dbox_body_state& b) {
    sb.set_v(i, b_v(b), b.vel[2]);
    sb.set_c(i, b_c(b), b.sweep[7]);
}

// flags of the compact per-body byte (s_bfl)
// (kBfPopped: the island search has walked the body's contacts, so every contact between it and
// a non-static body is already in an island)
enum { kBfAwake = 1, kBfActive = 2, kBfStatic = 4, kBfDynamic = 8, kBfVisited = 16, kBfMark = 32, kBfPopped = 64 };

// ------------------------------------------------------------ contact solver pieces (contacts/b2contactsolver.d)
// b2ContactSolver ctor (:244-329) for one contact; body indices are world-local.
DG void constraint_ctor(const Ctx& x, int ci, int b0, bool warm, float dtRatio, VC& vc, PC& pc) {
    const dbox_contact_state& c = x.ct[ci];
    const DFixture& fa = x.fx[c.fixture_a];
    const DFixture& fb = x.fx[c.fixture_b];
    const dbox_body_state& ba = x.bs[fa.body];
    const dbox_body_state& bb = x.bs[fb.body];
    int pointCount = c.point_count;
    vc.friction = c.friction;
    vc.restitution = c.restitution;
    vc.tangentSpeed = c.tangent_speed;
    vc.bodyA = fa.body - b0;
    vc.bodyB = fb.body - b0;
    vc.invMassA = ba.mass[1];
    vc.invMassB = bb.mass[1];
    vc.invIA = ba.mass[3];
    vc.invIB = bb.mass[3];
    vc.pointCount = pointCount;
    vc.K[0] = vc.K[1] = vc.K[2] = vc.K[3] = 0.0f;
    vc.NM[0] = vc.NM[1] = vc.NM[2] = vc.NM[3] = 0.0f;
    vc.normal = v2(0.0f, 0.0f);
    pc.bodyA = vc.bodyA;
    pc.bodyB = vc.bodyB;
    pc.invMassA = ba.mass[1];
    pc.invMassB = bb.mass[1];
    pc.lcA = b_lc(ba);
    pc.lcB = b_lc(bb);
    pc.invIA = ba.mass[3];
    pc.invIB = bb.mass[3];
    pc.localNormal = v2(c.local_normal[0], c.local_normal[1]);
    pc.localPoint = v2(c.local_point[0], c.local_point[1]);
    pc.pointCount = pointCount;
    pc.radiusA = fa.radius;
    pc.radiusB = fb.radius;
    pc.type = c.type;
#pragma unroll
    for (int j = 0; j < 2; ++j) {
        VPoint& p = vc.p[j];
        p.normalImpulse = 0.0f;
        p.tangentImpulse = 0.0f;
        if (j < pointCount && warm) {
            p.normalImpulse = dtRatio * c.points[j].normal_impulse;
            p.tangentImpulse = dtRatio * c.points[j].tangent_impulse;
        }
        p.rA = v2(0.0f, 0.0f);
        p.rB = v2(0.0f, 0.0f);
        p.normalMass = 0.0f;
        p.tangentMass = 0.0f;
        p.velocityBias = 0.0f;
        pc.localPoints[j] = j < pointCount ? v2(c.points[j].local_point[0], c.points[j].local_point[1]) : v2(0.0f, 0.0f);
    }
}

// InitializeVelocityConstraints (:338-450) for one contact
DG void constraint_init_velocity(VC& vc, const PC& pc, SB sb, float* sep = nullptr) {
    int pointCount = vc.pointCount;
    float mA = vc.invMassA, mB = vc.invMassB, iA = vc.invIA, iB = vc.invIB;
    float2 cA = sb.c(vc.bodyA), cB = sb.c(vc.bodyB);
    float aA = sb.a(vc.bodyA), aB = sb.a(vc.bodyB);
    float2 vA = sb.v(vc.bodyA), vB = sb.v(vc.bodyB);
    float wA = sb.w(vc.bodyA), wB = sb.w(vc.bodyB);
    Xf xfA, xfB;
    xfA.q = rot(aA);
    xfB.q = rot(aB);
    xfA.p = cA - mul(xfA.q, pc.lcA);
    xfB.p = cB - mul(xfB.q, pc.lcB);
    // b2WorldManifold.Initialize (b2collision.d:123-191)
    float2 normal = v2(0.0f, 0.0f);
    float2 points[2] = {v2(0.0f, 0.0f), v2(0.0f, 0.0f)};
    float radiusA = pc.radiusA, radiusB = pc.radiusB;
    if (pointCount > 0) {
        if (pc.type == kManifoldCircles) {
            normal = v2(1.0f, 0.0f);
            float2 pointA = mul(xfA, pc.localPoint);
            float2 pointB = mul(xfB, pc.localPoints[0]);
            if (dist_sq(pointA, pointB) > kEpsilon * kEpsilon) {
                normal = pointB - pointA;
                normalize(normal);
            }
            float2 ccA = pointA + radiusA * normal;
            float2 ccB = pointB - radiusB * normal;
            points[0] = 0.5f * (ccA + ccB);
            if (sep) sep[0] = dot(ccB - ccA, normal);
        } else if (pc.type == kManifoldFaceA) {
            normal = mul(xfA.q, pc.localNormal);
            float2 planePoint = mul(xfA, pc.localPoint);
#pragma unroll
            for (int i = 0; i < 2; ++i) {
                if (i < pointCount) {
                    float2 clipPoint = mul(xfB, pc.localPoints[i]);
                    float2 ccA = clipPoint + (radiusA - dot(clipPoint - planePoint, normal)) * normal;
                    float2 ccB = clipPoint - radiusB * normal;
                    points[i] = 0.5f * (ccA + ccB);
                    if (sep) sep[i] = dot(ccB - ccA, normal);
                }
            }
        } else {
            normal = mul(xfB.q, pc.localNormal);
            float2 planePoint = mul(xfB, pc.localPoint);
#pragma unroll
            for (int i = 0; i < 2; ++i) {
                if (i < pointCount) {
                    float2 clipPoint = mul(xfA, pc.localPoints[i]);
                    float2 ccB = clipPoint + (radiusB - dot(clipPoint - planePoint, normal)) * normal;
                    float2 ccA = clipPoint - radiusA * normal;
                    points[i] = 0.5f * (ccA + ccB);
                    if (sep) sep[i] = dot(ccA - ccB, normal);
                }
            }
            normal = -normal;
        }
    }
    vc.normal = normal;
#pragma unroll
    for (int j = 0; j < 2; ++j) {
        if (j >= pointCount) break;
        VPoint& p = vc.p[j];
        p.rA = points[j] - cA;
        p.rB = points[j] - cB;
        float rnA = cross(p.rA, normal);
        float rnB = cross(p.rB, normal);
        float kNormal = ((mA + mB) + (iA * rnA) * rnA) + (iB * rnB) * rnB;
        p.normalMass = kNormal > 0.0f ? fdiv(1.0f, kNormal) : 0.0f;
        float2 tangent = cross(normal, 1.0f);
        float rtA = cross(p.rA, tangent);
        float rtB = cross(p.rB, tangent);
        float kTangent = ((mA + mB) + (iA * rtA) * rtA) + (iB * rtB) * rtB;
        p.tangentMass = kTangent > 0.0f ? fdiv(1.0f, kTangent) : 0.0f;
        p.velocityBias = 0.0f;
        float vRel = dot(normal, ((vB + cross(wB, p.rB)) - vA) - cross(wA, p.rA));
        if (vRel < -kVelocityThreshold) p.velocityBias = -vc.restitution * vRel;
    }
    if (vc.pointCount == 2) {
        const VPoint& p1 = vc.p[0];
        const VPoint& p2 = vc.p[1];
        float rn1A = cross(p1.rA, normal), rn1B = cross(p1.rB, normal);
        float rn2A = cross(p2.rA, normal), rn2B = cross(p2.rB, normal);
        float k11 = ((mA + mB) + (iA * rn1A) * rn1A) + (iB * rn1B) * rn1B;
        float k22 = ((mA + mB) + (iA * rn2A) * rn2A) + (iB * rn2B) * rn2B;
        float k12 = ((mA + mB) + (iA * rn1A) * rn2A) + (iB * rn1B) * rn2B;
        if (k11 * k11 < 1000.0f * (k11 * k22 - k12 * k12)) {
            vc.K[0] = k11; vc.K[1] = k12; vc.K[2] = k12; vc.K[3] = k22;
            // b2Mat22.GetInverse (b2math.d:322-337)
            float a = vc.K[0], b = vc.K[2], cc = vc.K[1], d = vc.K[3];
            float det = a * d - b * cc;
            if (det != 0.0f) det = fdiv(1.0f, det);
            vc.NM[0] = det * d;
            vc.NM[2] = -det * b;
            vc.NM[1] = -det * cc;
            vc.NM[3] = det * a;
        } else {
            vc.pointCount = 1;
        }
    }
}

DG void warm_start(const VC& vc, SB sb) {                              // :452-490
    float mA = vc.invMassA, iA = vc.invIA, mB = vc.invMassB, iB = vc.invIB;
    float2 vA = sb.v(vc.bodyA), vB = sb.v(vc.bodyB);
    float wA = sb.w(vc.bodyA), wB = sb.w(vc.bodyB);
    float2 normal = vc.normal;
    float2 tangent = cross(normal, 1.0f);
#pragma unroll
    for (int j = 0; j < 2; ++j) {
        if (j >= vc.pointCount) break;
        const VPoint& p = vc.p[j];
        float2 P = p.normalImpulse * normal + p.tangentImpulse * tangent;
        wA -= iA * cross(p.rA, P);
        vA -= mA * P;
        wB += iB * cross(p.rB, P);
        vB += mB * P;
    }
    sb.set_v(vc.bodyA, vA, wA);
    sb.set_v(vc.bodyB, vB, wB);
}

DG void apply_block(float2& vA, float& wA, float2& vB, float& wB, float mA, float iA, float mB, float iB,
                    const VPoint& cp1, const VPoint& cp2, float2 normal, float2 d) {
    float2 P1 = d.x * normal;
    float2 P2 = d.y * normal;
    vA -= mA * (P1 + P2);
    wA -= iA * (cross(cp1.rA, P1) + cross(cp2.rA, P2));
    vB += mB * (P1 + P2);
    wB += iB * (cross(cp1.rB, P1) + cross(cp2.rB, P2));
}

// The velocities of the contact's two bodies in registers: loaded before a row picks its
// path, so the loads are in flight while the row's kind is tested.
struct BodyVel { float2 vA, vB; float wA, wB; };
DG BodyVel load_vel(SB sb, int a, int b) { BodyVel q; q.vA = sb.v(a); q.wA = sb.w(a); q.vB = sb.v(b); q.wB = sb.w(b); return q; }
DG void store_vel(SB sb, int a, int b, const BodyVel& q) { sb.set_v(a, q.vA, q.wA); sb.set_v(b, q.vB, q.wB); }

DG void solve_velocity(VC& vc, BodyVel& q) {                           // :492-772
    float mA = vc.invMassA, iA = vc.invIA, mB = vc.invMassB, iB = vc.invIB;
    int pointCount = vc.pointCount;
    float2 vA = q.vA, vB = q.vB;
    float wA = q.wA, wB = q.wB;
    float2 normal = vc.normal;
    float2 tangent = cross(normal, 1.0f);
    float friction = vc.friction;
#pragma unroll
    for (int j = 0; j < 2; ++j) {
        if (j >= pointCount) break;
        VPoint& p = vc.p[j];
        float2 dv = ((vB + cross(wB, p.rB)) - vA) - cross(wA, p.rA);
        float vt = dot(dv, tangent) - vc.tangentSpeed;
        float lambda = p.tangentMass * (-vt);
        float maxFriction = friction * p.normalImpulse;
        float newImpulse = bclamp(p.tangentImpulse + lambda, -maxFriction, maxFriction);
        lambda = newImpulse - p.tangentImpulse;
        p.tangentImpulse = newImpulse;
        float2 P = lambda * tangent;
        vA -= mA * P;
        wA -= iA * cross(p.rA, P);
        vB += mB * P;
        wB += iB * cross(p.rB, P);
    }
    if (pointCount == 1) {
        VPoint& p = vc.p[0];
        float2 dv = ((vB + cross(wB, p.rB)) - vA) - cross(wA, p.rA);
        float vn = dot(dv, normal);
        float lambda = -p.normalMass * (vn - p.velocityBias);
        float newImpulse = bmax(p.normalImpulse + lambda, 0.0f);
        lambda = newImpulse - p.normalImpulse;
        p.normalImpulse = newImpulse;
        float2 P = lambda * normal;
        vA -= mA * P;
        wA -= iA * cross(p.rA, P);
        vB += mB * P;
        wB += iB * cross(p.rB, P);
    } else {
        VPoint& cp1 = vc.p[0];
        VPoint& cp2 = vc.p[1];
        float2 a = v2(cp1.normalImpulse, cp2.normalImpulse);
        float2 dv1 = ((vB + cross(wB, cp1.rB)) - vA) - cross(wA, cp1.rA);
        float2 dv2 = ((vB + cross(wB, cp2.rB)) - vA) - cross(wA, cp2.rA);
        float vn1 = dot(dv1, normal);
        float vn2 = dot(dv2, normal);
        float2 b;
        b.x = vn1 - cp1.velocityBias;
        b.y = vn2 - cp2.velocityBias;
        float2 Ka = v2(vc.K[0] * a.x + vc.K[2] * a.y, vc.K[1] * a.x + vc.K[3] * a.y);
        b -= Ka;
        // The four cases of the 2x2 LCP (b2contactsolver.d:620-760) are evaluated side by side
        // and the first one that holds is applied, exactly as the sequential case chain does;
        // evaluating them all keeps the lanes of a level on one path.
        float2 x1 = -v2(vc.NM[0] * b.x + vc.NM[2] * b.y, vc.NM[1] * b.x + vc.NM[3] * b.y);
        bool c1 = x1.x >= 0.0f && x1.y >= 0.0f;
        float x2 = -cp1.normalMass * b.x;
        bool c2 = x2 >= 0.0f && vc.K[1] * x2 + b.y >= 0.0f;
        float x3 = -cp2.normalMass * b.y;
        bool c3 = x3 >= 0.0f && vc.K[2] * x3 + b.x >= 0.0f;
        bool c4 = b.x >= 0.0f && b.y >= 0.0f;
        float2 xx = c1 ? x1 : (c2 ? v2(x2, 0.0f) : (c3 ? v2(0.0f, x3) : v2(0.0f, 0.0f)));
        if (c1 || c2 || c3 || c4) {
            apply_block(vA, wA, vB, wB, mA, iA, mB, iB, cp1, cp2, normal, xx - a);
            cp1.normalImpulse = xx.x;
            cp2.normalImpulse = xx.y;
        }
    }
    q.vA = vA; q.wA = wA; q.vB = vB; q.wB = wB;
}
DG void solve_velocity(VC& vc, SB sb) {
    BodyVel q = load_vel(sb, vc.bodyA, vc.bodyB);
    solve_velocity(vc, q);
    store_vel(sb, vc.bodyA, vc.bodyB, q);
}

// solve_velocity for a contact with two points, with no branch inside: both friction points,
// then the block solver's four cases side by side; when no case holds, the velocities and
// impulses keep their values through selects instead of a skipped branch.  The same
// operations in the same order as solve_velocity, so the same bits; a branch costs tens of
// cycles on the dependent chain between levels, a select a few.
DG void solve_velocity_two(VC& vc, BodyVel& q) {
    float mA = vc.invMassA, iA = vc.invIA, mB = vc.invMassB, iB = vc.invIB;
    float2 vA = q.vA, vB = q.vB;
    float wA = q.wA, wB = q.wB;
    float2 normal = vc.normal;
    float2 tangent = cross(normal, 1.0f);
    float friction = vc.friction;
#pragma unroll
    for (int j = 0; j < 2; ++j) {
        VPoint& p = vc.p[j];
        float2 dv = ((vB + cross(wB, p.rB)) - vA) - cross(wA, p.rA);
        float vt = dot(dv, tangent) - vc.tangentSpeed;
        float lambda = p.tangentMass * (-vt);
        float maxFriction = friction * p.normalImpulse;
        float newImpulse = bclamp(p.tangentImpulse + lambda, -maxFriction, maxFriction);
        lambda = newImpulse - p.tangentImpulse;
        p.tangentImpulse = newImpulse;
        float2 P = lambda * tangent;
        vA -= mA * P;
        wA -= iA * cross(p.rA, P);
        vB += mB * P;
        wB += iB * cross(p.rB, P);
    }
    VPoint& cp1 = vc.p[0];
    VPoint& cp2 = vc.p[1];
    float2 a = v2(cp1.normalImpulse, cp2.normalImpulse);
    float2 dv1 = ((vB + cross(wB, cp1.rB)) - vA) - cross(wA, cp1.rA);
    float2 dv2 = ((vB + cross(wB, cp2.rB)) - vA) - cross(wA, cp2.rA);
    float vn1 = dot(dv1, normal);
    float vn2 = dot(dv2, normal);
    float2 b;
    b.x = vn1 - cp1.velocityBias;
    b.y = vn2 - cp2.velocityBias;
    float2 Ka = v2(vc.K[0] * a.x + vc.K[2] * a.y, vc.K[1] * a.x + vc.K[3] * a.y);
    b -= Ka;
    float2 x1 = -v2(vc.NM[0] * b.x + vc.NM[2] * b.y, vc.NM[1] * b.x + vc.NM[3] * b.y);
    bool c1 = x1.x >= 0.0f && x1.y >= 0.0f;
    float x2 = -cp1.normalMass * b.x;
    bool c2 = x2 >= 0.0f && vc.K[1] * x2 + b.y >= 0.0f;
    float x3 = -cp2.normalMass * b.y;
    bool c3 = x3 >= 0.0f && vc.K[2] * x3 + b.x >= 0.0f;
    bool c4 = b.x >= 0.0f && b.y >= 0.0f;
    float2 xx = c1 ? x1 : (c2 ? v2(x2, 0.0f) : (c3 ? v2(0.0f, x3) : v2(0.0f, 0.0f)));
    const bool any = c1 || c2 || c3 || c4;
    float2 vA2 = vA, vB2 = vB;
    float wA2 = wA, wB2 = wB;
    apply_block(vA2, wA2, vB2, wB2, mA, iA, mB, iB, cp1, cp2, normal, xx - a);
    vA.x = any ? vA2.x : vA.x;
    vA.y = any ? vA2.y : vA.y;
    wA = any ? wA2 : wA;
    vB.x = any ? vB2.x : vB.x;
    vB.y = any ? vB2.y : vB.y;
    wB = any ? wB2 : wB;
    cp1.normalImpulse = any ? xx.x : a.x;
    cp2.normalImpulse = any ? xx.y : a.y;
    q.vA = vA; q.wA = wA; q.vB = vB; q.wB = wB;
}

// ---- learned warm start: the 32 input features of a contact (after
// InitializeVelocityConstraints, before the warm start), in this order: normal (2); per point
// (0 then 1, zeros when absent): rA (2), rB (2), relative normal and tangent velocity, normal
// mass, tangent mass, velocity bias; inverse masses and inertias (4); friction, restitution,
// point count, separation of each point (2), gravity along the normal times dt, wA, wB.
DG void contact_features(const VC& vc, const float sep[2], int pointCount, SB sb, float2 gravity, float h, float* f) {
    float2 n = vc.normal, t = cross(n, 1.0f);
    float2 vA = sb.v(vc.bodyA), vB = sb.v(vc.bodyB);
    float wA = sb.w(vc.bodyA), wB = sb.w(vc.bodyB);
    f[0] = n.x;
    f[1] = n.y;
#pragma unroll
    for (int j = 0; j < 2; ++j) {
        float* q = f + 2 + 9 * j;
        const VPoint& p = vc.p[j];
        bool on = j < pointCount;
        float2 dv = ((vB + cross(wB, p.rB)) - vA) - cross(wA, p.rA);
        q[0] = on ? p.rA.x : 0.0f;
        q[1] = on ? p.rA.y : 0.0f;
        q[2] = on ? p.rB.x : 0.0f;
        q[3] = on ? p.rB.y : 0.0f;
        q[4] = on ? dot(dv, n) : 0.0f;
        q[5] = on ? dot(dv, t) : 0.0f;
        q[6] = on ? p.normalMass : 0.0f;
        q[7] = on ? p.tangentMass : 0.0f;
        q[8] = on ? p.velocityBias : 0.0f;
    }
    f[20] = vc.invMassA;
    f[21] = vc.invIA;
    f[22] = vc.invMassB;
    f[23] = vc.invIB;
    f[24] = vc.friction;
    f[25] = vc.restitution;
    f[26] = (float)pointCount;
    f[27] = pointCount > 0 ? sep[0] : 0.0f;
    f[28] = pointCount > 1 ? sep[1] : 0.0f;
    f[29] = dot(gravity, n) * h;
    f[30] = wA;
    f[31] = wB;
}

DG void store_impulses(const Ctx& x, const VRow& r) {                 // :774-787
    dbox_contact_state& c = x.ct[r.ids.w];
    c.points[0].normal_impulse = r.imp.x;
    c.points[0].tangent_impulse = r.imp.y;
    if ((r.ids.z & 0xff) > 1) {
        c.points[1].normal_impulse = r.imp.z;
        c.points[1].tangent_impulse = r.imp.w;
    }
}

// ------------------------------------------------------------ constraint rows
DG VRow pack_v(const VC& vc, int item) {
    VRow r;
    r.r0 = make_float4(vc.p[0].rA.x, vc.p[0].rA.y, vc.p[0].rB.x, vc.p[0].rB.y);
    r.r1 = make_float4(vc.p[1].rA.x, vc.p[1].rA.y, vc.p[1].rB.x, vc.p[1].rB.y);
    r.imp = make_float4(vc.p[0].normalImpulse, vc.p[0].tangentImpulse, vc.p[1].normalImpulse, vc.p[1].tangentImpulse);
    r.mass = make_float4(vc.p[0].normalMass, vc.p[0].tangentMass, vc.p[1].normalMass, vc.p[1].tangentMass);
    r.nb = make_float4(vc.normal.x, vc.normal.y, vc.p[0].velocityBias, vc.p[1].velocityBias);
    r.K = make_float4(vc.K[0], vc.K[1], vc.K[3], vc.friction);
    r.NM = make_float4(vc.NM[0], vc.NM[1], vc.NM[3], vc.tangentSpeed);
    r.inv = make_float4(vc.invMassA, vc.invIA, vc.invMassB, vc.invIB);
    r.ids = make_int4(vc.bodyA, vc.bodyB, vc.pointCount, item);
    return r;
}
DG VRow load_v(const VRow* p) {
    VRow r;
    r.r0 = p->r0; r.r1 = p->r1; r.imp = p->imp; r.mass = p->mass; r.nb = p->nb;
    r.K = p->K; r.NM = p->NM; r.inv = p->inv; r.ids = p->ids;
    return r;
}
DG VC unpack_v(const VRow& r) {
    VC vc;
    vc.p[0].rA = v2(r.r0.x, r.r0.y); vc.p[0].rB = v2(r.r0.z, r.r0.w);
    vc.p[1].rA = v2(r.r1.x, r.r1.y); vc.p[1].rB = v2(r.r1.z, r.r1.w);
    vc.p[0].normalImpulse = r.imp.x; vc.p[0].tangentImpulse = r.imp.y;
    vc.p[1].normalImpulse = r.imp.z; vc.p[1].tangentImpulse = r.imp.w;
    vc.p[0].normalMass = r.mass.x; vc.p[0].tangentMass = r.mass.y;
    vc.p[1].normalMass = r.mass.z; vc.p[1].tangentMass = r.mass.w;
    vc.normal = v2(r.nb.x, r.nb.y);
    vc.p[0].velocityBias = r.nb.z; vc.p[1].velocityBias = r.nb.w;
    vc.K[0] = r.K.x; vc.K[1] = r.K.y; vc.K[2] = r.K.y; vc.K[3] = r.K.z;
    vc.friction = r.K.w;
    vc.NM[0] = r.NM.x; vc.NM[1] = r.NM.y; vc.NM[2] = r.NM.y; vc.NM[3] = r.NM.z;
    vc.tangentSpeed = r.NM.w;
    vc.restitution = 0.0f;                       // only read while the row is built
    vc.invMassA = r.inv.x; vc.invIA = r.inv.y; vc.invMassB = r.inv.z; vc.invIB = r.inv.w;
    vc.bodyA = r.ids.x; vc.bodyB = r.ids.y; vc.pointCount = r.ids.z & 0xff;
    return vc;
}
DG PRow pack_p(const PC& pc, int island) {
    PRow r;
    r.lp = make_float4(pc.localPoints[0].x, pc.localPoints[0].y, pc.localPoints[1].x, pc.localPoints[1].y);
    r.ln = make_float4(pc.localNormal.x, pc.localNormal.y, pc.localPoint.x, pc.localPoint.y);
    r.lc = make_float4(pc.lcA.x, pc.lcA.y, pc.lcB.x, pc.lcB.y);
    r.inv = make_float4(pc.invMassA, pc.invIA, pc.invMassB, pc.invIB);
    r.rad = make_float4(pc.radiusA, pc.radiusB, 0.0f, 0.0f);
    r.ids = make_int4(pc.bodyA, pc.bodyB, pc.type | (pc.pointCount << 4), island);
    return r;
}
DG PRow load_p(const PRow* p) {
    PRow r;
    r.lp = p->lp; r.ln = p->ln; r.lc = p->lc; r.inv = p->inv; r.rad = p->rad; r.ids = p->ids;
    return r;
}
DG PC unpack_p(const PRow& r) {
    PC pc;
    pc.localPoints[0] = v2(r.lp.x, r.lp.y); pc.localPoints[1] = v2(r.lp.z, r.lp.w);
    pc.localNormal = v2(r.ln.x, r.ln.y); pc.localPoint = v2(r.ln.z, r.ln.w);
    pc.lcA = v2(r.lc.x, r.lc.y); pc.lcB = v2(r.lc.z, r.lc.w);
    pc.invMassA = r.inv.x; pc.invIA = r.inv.y; pc.invMassB = r.inv.z; pc.invIB = r.inv.w;
    pc.radiusA = r.rad.x; pc.radiusB = r.rad.y;
    pc.bodyA = r.ids.x; pc.bodyB = r.ids.y; pc.type = r.ids.z & 15; pc.pointCount = r.ids.z >> 4;
    return pc;
}

// SolvePositionConstraints / SolveTOIPositionConstraints for one contact (:73-242);
// returns the minimum separation seen over its points (0 if none below 0).
DG float solve_position(const PC& pc, SB sb, bool toi, int toiA, int toiB) {
    float mA, iA, mB, iB;
    if (!toi) { mA = pc.invMassA; iA = pc.invIA; mB = pc.invMassB; iB = pc.invIB; }
    else {
        mA = 0.0f; iA = 0.0f;
        if (pc.bodyA == toiA || pc.bodyA == toiB) { mA = pc.invMassA; iA = pc.invIA; }
        mB = 0.0f; iB = 0.0f;
        if (pc.bodyB == toiA || pc.bodyB == toiB) { mB = pc.invMassB; iB = pc.invIB; }
    }
    float2 cA = sb.c(pc.bodyA), cB = sb.c(pc.bodyB);
    float aA = sb.a(pc.bodyA), aB = sb.a(pc.bodyB);
    float minSep = 0.0f;
#pragma unroll
    for (int j = 0; j < 2; ++j) {
        if (j >= pc.pointCount) break;
        Xf xfA, xfB;
        xfA.q = rot(aA);
        xfB.q = rot(aB);
        xfA.p = cA - mul(xfA.q, pc.lcA);
        xfB.p = cB - mul(xfB.q, pc.lcB);
        // b2PositionSolverManifold.Initialize (:816-851)
        float2 normal, point;
        float separation;
        if (pc.type == kManifoldCircles) {
            float2 pointA = mul(xfA, pc.localPoint);
            float2 pointB = mul(xfB, pc.localPoints[0]);
            normal = pointB - pointA;
            normalize(normal);
            point = 0.5f * (pointA + pointB);
            separation = (dot(pointB - pointA, normal) - pc.radiusA) - pc.radiusB;
        } else {
            // e_faceA and e_faceB share one path: the reference face's transform is picked
            // first, and the normal is flipped for e_faceB
            bool faceA = pc.type == kManifoldFaceA;
            Xf xfN = faceA ? xfA : xfB, xfC = faceA ? xfB : xfA;
            normal = mul(xfN.q, pc.localNormal);
            float2 planePoint = mul(xfN, pc.localPoint);
            float2 clipPoint = mul(xfC, pc.localPoints[j]);
            separation = (dot(clipPoint - planePoint, normal) - pc.radiusA) - pc.radiusB;
            point = clipPoint;
            if (!faceA) normal = -normal;
        }
        float2 rA = point - cA;
        float2 rB = point - cB;
        minSep = bmin(minSep, separation);
        float C = bclamp((toi ? kToiBaumgarte : kBaumgarte) * (separation + kLinearSlop), -kMaxLinearCorrection, 0.0f);
        float rnA = cross(rA, normal);
        float rnB = cross(rB, normal);
        float K = ((mA + mB) + (iA * rnA) * rnA) + (iB * rnB) * rnB;
        float impulse = K > 0.0f ? fdiv(-C, K) : 0.0f;
        float2 P = impulse * normal;
        cA -= mA * P;
        aA -= iA * cross(rA, P);
        cB += mB * P;
        aB += iB * cross(rB, P);
    }
    sb.set_c(pc.bodyA, cA, aA);
    sb.set_c(pc.bodyB, cB, aB);
    return minSep;
}

// sin and cos on the binary32 path of dbox_sincosf alone (|x| <= 1024; zero handled the same way)
DG Rot rot_near(float x) {
    Rot q;
    dbox_trig::sincos_f32(x, &q.s, &q.c);
    if (x == 0.0f) { q.s = x; q.c = 1.0f; }
    return q;
}

// solve_position (non-TOI) for a polygon contact (e_faceA / e_faceB) with two points, with
// the rotations on the binary32 path only: one range test for the row replaces a rare-case
// branch inside each of its four rotations.  Returns false, with the bodies untouched, when
// an angle was outside |a| <= 1024 (or not finite); the caller then runs solve_position,
// which gives the row's true result.  Otherwise the same operations in the same order as
// solve_position, so the same bits.
DG bool solve_position_two(const PC& pc, float2& cA_io, float& aA_io, float2& cB_io, float& aB_io, float& minSepOut) {
    const float mA = pc.invMassA, iA = pc.invIA, mB = pc.invMassB, iB = pc.invIB;
    float2 cA = cA_io, cB = cB_io;
    float aA = aA_io, aB = aB_io;
    const bool faceA = pc.type == kManifoldFaceA;
    float minSep = 0.0f;
    bool near = true;
#pragma unroll
    for (int j = 0; j < 2; ++j) {
        near = near && fabsf(aA) <= 1024.0f && fabsf(aB) <= 1024.0f;
        Xf xfA, xfB;
        xfA.q = rot_near(aA);
        xfB.q = rot_near(aB);
        xfA.p = cA - mul(xfA.q, pc.lcA);
        xfB.p = cB - mul(xfB.q, pc.lcB);
        Xf xfN = faceA ? xfA : xfB, xfC = faceA ? xfB : xfA;
        float2 normal = mul(xfN.q, pc.localNormal);
        float2 planePoint = mul(xfN, pc.localPoint);
        float2 clipPoint = mul(xfC, pc.localPoints[j]);
        float separation = (dot(clipPoint - planePoint, normal) - pc.radiusA) - pc.radiusB;
        float2 point = clipPoint;
        if (!faceA) normal = -normal;
        float2 rA = point - cA;
        float2 rB = point - cB;
        minSep = bmin(minSep, separation);
        float C = bclamp(kBaumgarte * (separation + kLinearSlop), -kMaxLinearCorrection, 0.0f);
        float rnA = cross(rA, normal);
        float rnB = cross(rB, normal);
        float K = ((mA + mB) + (iA * rnA) * rnA) + (iB * rnB) * rnB;
        float impulse = K > 0.0f ? fdiv(-C, K) : 0.0f;
        float2 P = impulse * normal;
        cA -= mA * P;
        aA -= iA * cross(rA, P);
        cB += mB * P;
        aB += iB * cross(rB, P);
    }
    cA_io = cA; aA_io = aA; cB_io = cB; aB_io = aB;
    minSepOut = minSep;
    return near;
}

// one position row of SolvePositionConstraints: the two-point polygon path when it applies
// (the bodies' positions are loaded before the row's kind is tested)
DG float solve_position_row(const PC& pc, SB sb) {
    float2 cA = sb.c(pc.bodyA), cB = sb.c(pc.bodyB);
    float aA = sb.a(pc.bodyA), aB = sb.a(pc.bodyB);
    float ms;
    if (pc.pointCount == 2 && pc.type != kManifoldCircles && solve_position_two(pc, cA, aA, cB, aB, ms)) {
        sb.set_c(pc.bodyA, cA, aA);
        sb.set_c(pc.bodyB, cB, aB);
        return ms;
    }
    return solve_position(pc, sb, false, -1, -1);
}

DG float3 solve33(const float* m, float3 b) {                            // b2math.d:388-399
    float3 ex = make_float3(m[0], m[1], m[2]), ey = make_float3(m[3], m[4], m[5]), ez = make_float3(m[6], m[7], m[8]);
    auto cr = [](float3 a, float3 c) { return make_float3(a.y * c.z - a.z * c.y, a.z * c.x - a.x * c.z, a.x * c.y - a.y * c.x); };
    auto dt3 = [](float3 a, float3 c) { return (a.x * c.x + a.y * c.y) + a.z * c.z; };
    float det = dt3(ex, cr(ey, ez));
    if (det != 0.0f) det = fdiv(1.0f, det);
    float3 r;
    r.x = det * dt3(b, cr(ey, ez));
    r.y = det * dt3(ex, cr(b, ez));
    r.z = det * dt3(ex, cr(ey, b));
    return r;
}
DG float2 solve22(const float* m, float2 b) {                            // b2math.d:402-415
    float a11 = m[0], a12 = m[3], a21 = m[1], a22 = m[4];
    float det = a11 * a22 - a12 * a21;
    if (det != 0.0f) det = fdiv(1.0f, det);
    return v2(det * (a22 * b.x - a12 * b.y), det * (a11 * b.y - a21 * b.x));
}

// ------------------------------------------------------------ distance joint (joints/b2distancejoint.d:211-372)
__device__ __noinline__ void distance_init(const Ctx& x, int ji, int b0, SB sb, bool warm, float dtRatio) {
    DJoint& j = x.jt[ji];
    const dbox_body_state& ba = x.bs[j.body_a];
    const dbox_body_state& bb = x.bs[j.body_b];
    int la = j.body_a - b0, lb = j.body_b - b0;
    j.lcA = b_lc(ba);
    j.lcB = b_lc(bb);
    j.invMassA = ba.mass[1];
    j.invMassB = bb.mass[1];
    j.invIA = ba.mass[3];
    j.invIB = bb.mass[3];
    float2 cA = sb.c(la), cB = sb.c(lb);
    float aA = sb.a(la), aB = sb.a(lb);
    float2 vA = sb.v(la), vB = sb.v(lb);
    float wA = sb.w(la), wB = sb.w(lb);
    Rot qA = rot(aA), qB = rot(aB);
    j.rA = mul(qA, j.local_anchor_a - j.lcA);
    j.rB = mul(qB, j.local_anchor_b - j.lcB);
    float2 u = ((cB + j.rB) - cA) - j.rA;
    float len = length(u);                                              // singularity: u = 0 below linearSlop
    if (len > kLinearSlop) u *= fdiv(1.0f, len);
    else u = v2(0.0f, 0.0f);
    j.u = u;
    float crAu = cross(j.rA, u), crBu = cross(j.rB, u);
    float invMass = ((j.invMassA + (j.invIA * crAu) * crAu) + j.invMassB) + (j.invIB * crBu) * crBu;
    float mass = invMass != 0.0f ? fdiv(1.0f, invMass) : 0.0f;
    if (j.frequency_hz > 0.0f) {
        float C = len - j.length;
        float omega = (2.0f * kPi) * j.frequency_hz;
        float d = ((2.0f * mass) * j.damping_ratio) * omega;
        float k = (mass * omega) * omega;
        float h = x.dt;
        float gamma = h * (d + h * k);
        gamma = gamma != 0.0f ? fdiv(1.0f, gamma) : 0.0f;
        j.gamma = gamma;
        j.bias = ((C * h) * k) * gamma;
        invMass += gamma;
        mass = invMass != 0.0f ? fdiv(1.0f, invMass) : 0.0f;
    } else {
        j.gamma = 0.0f;
        j.bias = 0.0f;
    }
    j.mass[0] = mass;
    if (warm) {
        j.impulse[0] *= dtRatio;
        float2 P = j.impulse[0] * u;
        vA -= j.invMassA * P;
        wA -= j.invIA * cross(j.rA, P);
        vB += j.invMassB * P;
        wB += j.invIB * cross(j.rB, P);
    } else {
        j.impulse[0] = 0.0f;
    }
    sb.set_v(la, vA, wA);
    sb.set_v(lb, vB, wB);
}

DG void distance_solve_velocity(DJoint& j, int la, int lb, SB sb) {
    float2 vA = sb.v(la), vB = sb.v(lb);
    float wA = sb.w(la), wB = sb.w(lb);
    float2 vpA = vA + cross(wA, j.rA);
    float2 vpB = vB + cross(wB, j.rB);
    float Cdot = dot(j.u, vpB - vpA);
    float impulse = -j.mass[0] * ((Cdot + j.bias) + j.gamma * j.impulse[0]);
    j.impulse[0] += impulse;
    float2 P = impulse * j.u;
    vA -= j.invMassA * P;
    wA -= j.invIA * cross(j.rA, P);
    vB += j.invMassB * P;
    wB += j.invIB * cross(j.rB, P);
    sb.set_v(la, vA, wA);
    sb.set_v(lb, vB, wB);
}

__device__ __noinline__ bool distance_solve_position(const DJoint& j, int la, int lb, SB sb) {
    if (j.frequency_hz > 0.0f) return true;                            // soft: no position correction
    float2 cA = sb.c(la), cB = sb.c(lb);
    float aA = sb.a(la), aB = sb.a(lb);
    Rot qA = rot(aA), qB = rot(aB);
    float2 rA = mul(qA, j.local_anchor_a - j.lcA);
    float2 rB = mul(qB, j.local_anchor_b - j.lcB);
    float2 u = ((cB + rB) - cA) - rA;
    float len = normalize(u);
    float C = bclamp(len - j.length, -kMaxLinearCorrection, kMaxLinearCorrection);
    float impulse = -j.mass[0] * C;
    float2 P = impulse * u;
    cA -= j.invMassA * P;
    aA -= j.invIA * cross(rA, P);
    cB += j.invMassB * P;
    aB += j.invIB * cross(rB, P);
    sb.set_c(la, cA, aA);
    sb.set_c(lb, cB, aB);
    return babs(C) < kLinearSlop;
}

// ------------------------------------------------------------ rope joint (joints/b2ropejoint.d:165-317)
__device__ __noinline__ void rope_init(const Ctx& x, int ji, int b0, SB sb, bool warm, float dtRatio) {
    DJoint& j = x.jt[ji];
    const dbox_body_state& ba = x.bs[j.body_a];
    const dbox_body_state& bb = x.bs[j.body_b];
    int la = j.body_a - b0, lb = j.body_b - b0;
    j.lcA = b_lc(ba);
    j.lcB = b_lc(bb);
    j.invMassA = ba.mass[1];
    j.invMassB = bb.mass[1];
    j.invIA = ba.mass[3];
    j.invIB = bb.mass[3];
    float2 cA = sb.c(la), cB = sb.c(lb);
    float aA = sb.a(la), aB = sb.a(lb);
    float2 vA = sb.v(la), vB = sb.v(lb);
    float wA = sb.w(la), wB = sb.w(lb);
    Rot qA = rot(aA), qB = rot(aB);
    j.rA = mul(qA, j.local_anchor_a - j.lcA);
    j.rB = mul(qB, j.local_anchor_b - j.lcB);
    float2 u = ((cB + j.rB) - cA) - j.rA;
    j.cur_length = length(u);
    float C = j.cur_length - j.length;
    j.limit_state = C > 0.0f ? 2 : 0;                                  // at upper limit / inactive
    if (j.cur_length > kLinearSlop) {
        u *= fdiv(1.0f, j.cur_length);
    } else {
        j.u = v2(0.0f, 0.0f);
        j.mass[0] = 0.0f;
        j.impulse[0] = 0.0f;
        return;
    }
    j.u = u;
    float crA = cross(j.rA, u), crB = cross(j.rB, u);
    float invMass = ((j.invMassA + (j.invIA * crA) * crA) + j.invMassB) + (j.invIB * crB) * crB;
    j.mass[0] = invMass != 0.0f ? fdiv(1.0f, invMass) : 0.0f;
    if (warm) {
        j.impulse[0] *= dtRatio;
        float2 P = j.impulse[0] * u;
        vA -= j.invMassA * P;
        wA -= j.invIA * cross(j.rA, P);
        vB += j.invMassB * P;
        wB += j.invIB * cross(j.rB, P);
    } else {
        j.impulse[0] = 0.0f;
    }
    sb.set_v(la, vA, wA);
    sb.set_v(lb, vB, wB);
}

DG void rope_solve_velocity(const Ctx& x, DJoint& j, int la, int lb, SB sb) {
    float2 vA = sb.v(la), vB = sb.v(lb);
    float wA = sb.w(la), wB = sb.w(lb);
    float2 vpA = vA + cross(wA, j.rA);
    float2 vpB = vB + cross(wB, j.rB);
    float C = j.cur_length - j.length;
    float Cdot = dot(j.u, vpB - vpA);
    if (C < 0.0f) Cdot += x.inv_dt * C;                                 // predictive constraint
    float impulse = -j.mass[0] * Cdot;
    float oldImpulse = j.impulse[0];
    j.impulse[0] = bmin(0.0f, j.impulse[0] + impulse);
    impulse = j.impulse[0] - oldImpulse;
    float2 P = impulse * j.u;
    vA -= j.invMassA * P;
    wA -= j.invIA * cross(j.rA, P);
    vB += j.invMassB * P;
    wB += j.invIB * cross(j.rB, P);
    sb.set_v(la, vA, wA);
    sb.set_v(lb, vB, wB);
}

__device__ __noinline__ bool rope_solve_position(const DJoint& j, int la, int lb, SB sb) {
    float2 cA = sb.c(la), cB = sb.c(lb);
    float aA = sb.a(la), aB = sb.a(lb);
    Rot qA = rot(aA), qB = rot(aB);
    float2 rA = mul(qA, j.local_anchor_a - j.lcA);
    float2 rB = mul(qB, j.local_anchor_b - j.lcB);
    float2 u = ((cB + rB) - cA) - rA;
    float len = normalize(u);
    float C = bclamp(len - j.length, 0.0f, kMaxLinearCorrection);
    float impulse = -j.mass[0] * C;
    float2 P = impulse * u;
    cA -= j.invMassA * P;
    aA -= j.invIA * cross(rA, P);
    cB += j.invMassB * P;
    aB += j.invIB * cross(rB, P);
    sb.set_c(la, cA, aA);
    sb.set_c(lb, cB, aB);
    return len - j.length < kLinearSlop;
}

// ------------------------------------------------------------ weld joint (joints/b2weldjoint.d:196-444)
// b2Mat33 in the joint's mass[9] layout: ex.x ex.y ex.z ey.x ey.y ey.z ez.x ez.y ez.z
DG void weld_k(float* K, float mA, float mB, float iA, float iB, float2 ra, float2 rb) {
    K[0] = ((mA + mB) + (ra.y * ra.y) * iA) + (rb.y * rb.y) * iB;       // ex.x
    K[3] = ((-ra.y) * ra.x) * iA - (rb.y * rb.x) * iB;                  // ey.x
    K[6] = (-ra.y) * iA - rb.y * iB;                                    // ez.x
    K[1] = K[3];                                                        // ex.y
    K[4] = ((mA + mB) + (ra.x * ra.x) * iA) + (rb.x * rb.x) * iB;       // ey.y
    K[7] = ra.x * iA + rb.x * iB;                                       // ez.y
    K[2] = K[6];                                                        // ex.z
    K[5] = K[7];                                                        // ey.z
    K[8] = iA + iB;                                                     // ez.z
}
DG void inverse22(const float* K, float* M) {                             // b2math.d:419-440
    float a = K[0], b = K[3], c = K[1], d = K[4];
    float det = a * d - b * c;
    if (det != 0.0f) det = fdiv(1.0f, det);
    M[0] = det * d;
    M[3] = -det * b;
    M[2] = 0.0f;
    M[1] = -det * c;
    M[4] = det * a;
    M[5] = 0.0f;
    M[6] = 0.0f;
    M[7] = 0.0f;
    M[8] = 0.0f;
}
DG void sym_inverse33(const float* K, float* M) {                        // b2math.d:442-465
    float3 ex = make_float3(K[0], K[1], K[2]), ey = make_float3(K[3], K[4], K[5]), ez = make_float3(K[6], K[7], K[8]);
    float3 c = make_float3(ey.y * ez.z - ey.z * ez.y, ey.z * ez.x - ey.x * ez.z, ey.x * ez.y - ey.y * ez.x);
    float det = (ex.x * c.x + ex.y * c.y) + ex.z * c.z;
    if (det != 0.0f) det = fdiv(1.0f, det);
    float a11 = ex.x, a12 = ey.x, a13 = ez.x;
    float a22 = ey.y, a23 = ez.y;
    float a33 = ez.z;
    M[0] = det * (a22 * a33 - a23 * a23);
    M[1] = det * (a13 * a23 - a12 * a33);
    M[2] = det * (a12 * a23 - a13 * a22);
    M[3] = M[1];
    M[4] = det * (a11 * a33 - a13 * a13);
    M[5] = det * (a13 * a12 - a11 * a23);
    M[6] = M[2];
    M[7] = M[5];
    M[8] = det * (a11 * a22 - a12 * a12);
}

__device__ __noinline__ void weld_init(const Ctx& x, int ji, int b0, SB sb, bool warm, float dtRatio) {
    DJoint& j = x.jt[ji];
    const dbox_body_state& ba = x.bs[j.body_a];
    const dbox_body_state& bb = x.bs[j.body_b];
    int la = j.body_a - b0, lb = j.body_b - b0;
    j.lcA = b_lc(ba);
    j.lcB = b_lc(bb);
    j.invMassA = ba.mass[1];
    j.invMassB = bb.mass[1];
    j.invIA = ba.mass[3];
    j.invIB = bb.mass[3];
    float aA = sb.a(la), aB = sb.a(lb);
    float2 vA = sb.v(la), vB = sb.v(lb);
    float wA = sb.w(la), wB = sb.w(lb);
    Rot qA = rot(aA), qB = rot(aB);
    j.rA = mul(qA, j.local_anchor_a - j.lcA);
    j.rB = mul(qB, j.local_anchor_b - j.lcB);
    const float mA = j.invMassA, mB = j.invMassB, iA = j.invIA, iB = j.invIB;
    float K[9];
    weld_k(K, mA, mB, iA, iB, j.rA, j.rB);
    if (j.frequency_hz > 0.0f) {
        inverse22(K, j.mass);
        float invM = iA + iB;
        float m = invM > 0.0f ? fdiv(1.0f, invM) : 0.0f;
        float C = (aB - aA) - j.reference_angle;
        float omega = (2.0f * kPi) * j.frequency_hz;
        float d = ((2.0f * m) * j.damping_ratio) * omega;
        float k = (m * omega) * omega;
        float h = x.dt;
        float gamma = h * (d + h * k);
        gamma = gamma != 0.0f ? fdiv(1.0f, gamma) : 0.0f;
        j.gamma = gamma;
        j.bias = ((C * h) * k) * gamma;
        invM += gamma;
        j.mass[8] = invM != 0.0f ? fdiv(1.0f, invM) : 0.0f;
    } else if (K[8] == 0.0f) {
        inverse22(K, j.mass);
        j.gamma = 0.0f;
        j.bias = 0.0f;
    } else {
        sym_inverse33(K, j.mass);
        j.gamma = 0.0f;
        j.bias = 0.0f;
    }
    if (warm) {
        j.impulse[0] *= dtRatio; j.impulse[1] *= dtRatio; j.impulse[2] *= dtRatio;
        float2 P = v2(j.impulse[0], j.impulse[1]);
        vA -= mA * P;
        wA -= iA * (cross(j.rA, P) + j.impulse[2]);
        vB += mB * P;
        wB += iB * (cross(j.rB, P) + j.impulse[2]);
    } else {
        j.impulse[0] = 0.0f; j.impulse[1] = 0.0f; j.impulse[2] = 0.0f;
    }
    sb.set_v(la, vA, wA);
    sb.set_v(lb, vB, wB);
}

__device__ __noinline__ void weld_solve_velocity(DJoint& j, int la, int lb, SB sb) {
    float2 vA = sb.v(la), vB = sb.v(lb);
    float wA = sb.w(la), wB = sb.w(lb);
    const float mA = j.invMassA, mB = j.invMassB, iA = j.invIA, iB = j.invIB;
    const float* M = j.mass;
    if (j.frequency_hz > 0.0f) {
        float Cdot2 = wB - wA;
        float impulse2 = -M[8] * ((Cdot2 + j.bias) + j.gamma * j.impulse[2]);
        j.impulse[2] += impulse2;
        wA -= iA * impulse2;
        wB += iB * impulse2;
        float2 Cdot1 = ((vB + cross(wB, j.rB)) - vA) - cross(wA, j.rA);
        float2 impulse1 = -v2(M[0] * Cdot1.x + M[3] * Cdot1.y, M[1] * Cdot1.x + M[4] * Cdot1.y);
        j.impulse[0] += impulse1.x;
        j.impulse[1] += impulse1.y;
        float2 P = impulse1;
        vA -= mA * P;
        wA -= iA * cross(j.rA, P);
        vB += mB * P;
        wB += iB * cross(j.rB, P);
    } else {
        float2 Cdot1 = ((vB + cross(wB, j.rB)) - vA) - cross(wA, j.rA);
        float Cdot2 = wB - wA;
        float3 imp = make_float3(-((Cdot1.x * M[0] + Cdot1.y * M[3]) + Cdot2 * M[6]),
                                 -((Cdot1.x * M[1] + Cdot1.y * M[4]) + Cdot2 * M[7]),
                                 -((Cdot1.x * M[2] + Cdot1.y * M[5]) + Cdot2 * M[8]));
        j.impulse[0] += imp.x;
        j.impulse[1] += imp.y;
        j.impulse[2] += imp.z;
        float2 P = v2(imp.x, imp.y);
        vA -= mA * P;
        wA -= iA * (cross(j.rA, P) + imp.z);
        vB += mB * P;
        wB += iB * (cross(j.rB, P) + imp.z);
    }
    sb.set_v(la, vA, wA);
    sb.set_v(lb, vB, wB);
}

__device__ __noinline__ bool weld_solve_position(const DJoint& j, int la, int lb, SB sb) {
    float2 cA = sb.c(la), cB = sb.c(lb);
    float aA = sb.a(la), aB = sb.a(lb);
    Rot qA = rot(aA), qB = rot(aB);
    const float mA = j.invMassA, mB = j.invMassB, iA = j.invIA, iB = j.invIB;
    float2 rA = mul(qA, j.local_anchor_a - j.lcA);
    float2 rB = mul(qB, j.local_anchor_b - j.lcB);
    float positionError, angularError;
    float K[9];
    weld_k(K, mA, mB, iA, iB, rA, rB);
    if (j.frequency_hz > 0.0f) {
        float2 C1 = ((cB + rB) - cA) - rA;
        positionError = length(C1);
        angularError = 0.0f;
        float2 P = -solve22(K, C1);
        cA -= mA * P;
        aA -= iA * cross(rA, P);
        cB += mB * P;
        aB += iB * cross(rB, P);
    } else {
        float2 C1 = ((cB + rB) - cA) - rA;
        float C2 = (aB - aA) - j.reference_angle;
        positionError = length(C1);
        angularError = babs(C2);
        float3 imp;
        if (K[8] > 0.0f) {
            float3 r = solve33(K, make_float3(C1.x, C1.y, C2));
            imp = make_float3(-r.x, -r.y, -r.z);
        } else {
            float2 r = solve22(K, C1);
            imp = make_float3(-r.x, -r.y, 0.0f);
        }
        float2 P = v2(imp.x, imp.y);
        cA -= mA * P;
        aA -= iA * (cross(rA, P) + imp.z);
        cB += mB * P;
        aB += iB * (cross(rB, P) + imp.z);
    }
    sb.set_c(la, cA, aA);
    sb.set_c(lb, cB, aB);
    return positionError <= kLinearSlop && angularError <= kAngularSlop;
}

// ------------------------------------------------------------ friction and motor joints
// b2FrictionJoint (joints/b2frictionjoint.d:178-315), b2MotorJoint (joints/b2motorjoint.d:223-366):
// a 2x2 linear and a 1x1 angular block with force / torque caps; the motor's anchors are the
// bodies' origins and it drives towards its offset with a correction factor
__device__ __noinline__ void friction_motor_init(const Ctx& x, int ji, int b0, SB sb, bool warm, float dtRatio) {
    DJoint& j = x.jt[ji];
    const dbox_body_state& ba = x.bs[j.body_a];
    const dbox_body_state& bb = x.bs[j.body_b];
    int la = j.body_a - b0, lb = j.body_b - b0;
    j.lcA = b_lc(ba);
    j.lcB = b_lc(bb);
    j.invMassA = ba.mass[1];
    j.invMassB = bb.mass[1];
    j.invIA = ba.mass[3];
    j.invIB = bb.mass[3];
    float2 cA = sb.c(la), cB = sb.c(lb);
    float aA = sb.a(la), aB = sb.a(lb);
    float2 vA = sb.v(la), vB = sb.v(lb);
    float wA = sb.w(la), wB = sb.w(lb);
    Rot qA = rot(aA), qB = rot(aB);
    const bool motor = j.type == kMotorJoint;
    if (motor) {
        j.rA = mul(qA, -j.lcA);
        j.rB = mul(qB, -j.lcB);
    } else {
        j.rA = mul(qA, j.local_anchor_a - j.lcA);
        j.rB = mul(qB, j.local_anchor_b - j.lcB);
    }
    const float mA = j.invMassA, mB = j.invMassB, iA = j.invIA, iB = j.invIB;
    const float2 rA = j.rA, rB = j.rB;
    float k11 = ((mA + mB) + (iA * rA.y) * rA.y) + (iB * rB.y) * rB.y;
    float k21 = ((-iA) * rA.x) * rA.y - (iB * rB.x) * rB.y;
    float k22 = ((mA + mB) + (iA * rA.x) * rA.x) + (iB * rB.x) * rB.x;
    float det = k11 * k22 - k21 * k21;                                  // b2Mat22.GetInverse (b2math.d:322-337)
    if (det != 0.0f) det = fdiv(1.0f, det);
    j.mass[0] = det * k22;
    j.mass[3] = -det * k21;
    j.mass[1] = -det * k21;
    j.mass[4] = det * k11;
    float am = iA + iB;
    if (am > 0.0f) am = fdiv(1.0f, am);
    j.angular_mass = am;
    if (motor) {
        j.linear_error = (((cB + rB) - cA) - rA) - mul(qA, j.linear_offset);
        j.angular_error = (aB - aA) - j.angular_offset;
    }
    if (warm) {
        j.impulse[0] *= dtRatio; j.impulse[1] *= dtRatio; j.impulse[2] *= dtRatio;
        float2 P = v2(j.impulse[0], j.impulse[1]);
        vA -= mA * P;
        wA -= iA * (cross(rA, P) + j.impulse[2]);
        vB += mB * P;
        wB += iB * (cross(rB, P) + j.impulse[2]);
    } else {
        j.impulse[0] = 0.0f; j.impulse[1] = 0.0f; j.impulse[2] = 0.0f;
    }
    sb.set_v(la, vA, wA);
    sb.set_v(lb, vB, wB);
}

__device__ __noinline__ void friction_motor_solve_velocity(const Ctx& x, DJoint& j, int la, int lb, SB sb) {
    float2 vA = sb.v(la), vB = sb.v(lb);
    float wA = sb.w(la), wB = sb.w(lb);
    const float mA = j.invMassA, mB = j.invMassB, iA = j.invIA, iB = j.invIB;
    const float h = x.dt, inv_h = x.inv_dt;
    const bool motor = j.type == kMotorJoint;
    {
        float Cdot = wB - wA;
        if (motor) Cdot = Cdot + (inv_h * j.correction_factor) * j.angular_error;
        float impulse = -j.angular_mass * Cdot;
        float oldImpulse = j.impulse[2];
        float maxImpulse = h * j.max_torque;
        j.impulse[2] = bclamp(j.impulse[2] + impulse, -maxImpulse, maxImpulse);
        impulse = j.impulse[2] - oldImpulse;
        wA -= iA * impulse;
        wB += iB * impulse;
    }
    {
        float2 Cdot = ((vB + cross(wB, j.rB)) - vA) - cross(wA, j.rA);
        if (motor) Cdot = Cdot + (inv_h * j.correction_factor) * j.linear_error;
        float2 impulse = -v2(j.mass[0] * Cdot.x + j.mass[3] * Cdot.y, j.mass[1] * Cdot.x + j.mass[4] * Cdot.y);
        float2 oldImpulse = v2(j.impulse[0], j.impulse[1]);
        float2 li = v2(j.impulse[0] + impulse.x, j.impulse[1] + impulse.y);
        float maxImpulse = h * j.max_force;
        if (li.x * li.x + li.y * li.y > maxImpulse * maxImpulse) {
            normalize(li);
            li *= maxImpulse;
        }
        j.impulse[0] = li.x;
        j.impulse[1] = li.y;
        impulse = li - oldImpulse;
        vA -= mA * impulse;
        wA -= iA * cross(j.rA, impulse);
        vB += mB * impulse;
        wB += iB * cross(j.rB, impulse);
    }
    sb.set_v(la, vA, wA);
    sb.set_v(lb, vB, wB);
}

// ------------------------------------------------------------ wheel joint (joints/b2wheeljoint.d:302-553)
__device__ __noinline__ void wheel_init(const Ctx& x, int ji, int b0, SB sb, bool warm, float dtRatio) {
    DJoint& j = x.jt[ji];
    const dbox_body_state& ba = x.bs[j.body_a];
    const dbox_body_state& bb = x.bs[j.body_b];
    int la = j.body_a - b0, lb = j.body_b - b0;
    j.lcA = b_lc(ba);
    j.lcB = b_lc(bb);
    j.invMassA = ba.mass[1];
    j.invMassB = bb.mass[1];
    j.invIA = ba.mass[3];
    j.invIB = bb.mass[3];
    const float mA = j.invMassA, mB = j.invMassB, iA = j.invIA, iB = j.invIB;
    float2 cA = sb.c(la), cB = sb.c(lb);
    float aA = sb.a(la), aB = sb.a(lb);
    float2 vA = sb.v(la), vB = sb.v(lb);
    float wA = sb.w(la), wB = sb.w(lb);
    Rot qA = rot(aA), qB = rot(aB);
    float2 rA = mul(qA, j.local_anchor_a - j.lcA);
    float2 rB = mul(qB, j.local_anchor_b - j.lcB);
    float2 d = ((cB + rB) - cA) - rA;
    j.ay = mul(qA, j.local_axis_y);                                     // point to line
    j.sAy = cross(d + rA, j.ay);
    j.sBy = cross(rB, j.ay);
    float m = ((mA + mB) + (iA * j.sAy) * j.sAy) + (iB * j.sBy) * j.sBy;
    if (m > 0.0f) m = fdiv(1.0f, m);
    j.mass[0] = m;
    j.spring_mass = 0.0f;                                               // spring
    j.bias = 0.0f;
    j.gamma = 0.0f;
    if (j.frequency_hz > 0.0f) {
        j.ax = mul(qA, j.local_axis_x);
        j.sAx = cross(d + rA, j.ax);
        j.sBx = cross(rB, j.ax);
        float invMass = ((mA + mB) + (iA * j.sAx) * j.sAx) + (iB * j.sBx) * j.sBx;
        if (invMass > 0.0f) {
            float sm = fdiv(1.0f, invMass);
            float C = dot(d, j.ax);
            float omega = (2.0f * kPi) * j.frequency_hz;
            float d2 = ((2.0f * sm) * j.damping_ratio) * omega;
            float k = (sm * omega) * omega;
            float h = x.dt;
            float gamma = h * (d2 + h * k);
            if (gamma > 0.0f) gamma = fdiv(1.0f, gamma);
            j.gamma = gamma;
            j.bias = ((C * h) * k) * gamma;
            sm = invMass + gamma;
            if (sm > 0.0f) sm = fdiv(1.0f, sm);
            j.spring_mass = sm;
        }
    } else {
        j.impulse[1] = 0.0f;
    }
    if (j.enable_motor) {                                               // rotational motor
        float mm = iA + iB;
        if (mm > 0.0f) mm = fdiv(1.0f, mm);
        j.motor_mass = mm;
    } else {
        j.motor_mass = 0.0f;
        j.motor_impulse = 0.0f;
    }
    if (warm) {
        j.impulse[0] *= dtRatio;
        j.impulse[1] *= dtRatio;
        j.motor_impulse *= dtRatio;
        float2 P = j.impulse[0] * j.ay + j.impulse[1] * j.ax;
        float LA = (j.impulse[0] * j.sAy + j.impulse[1] * j.sAx) + j.motor_impulse;
        float LB = (j.impulse[0] * j.sBy + j.impulse[1] * j.sBx) + j.motor_impulse;
        vA -= mA * P;
        wA -= iA * LA;
        vB += mB * P;
        wB += iB * LB;
    } else {
        j.impulse[0] = 0.0f;
        j.impulse[1] = 0.0f;
        j.motor_impulse = 0.0f;
    }
    sb.set_v(la, vA, wA);
    sb.set_v(lb, vB, wB);
}

__device__ __noinline__ void wheel_solve_velocity(const Ctx& x, DJoint& j, int la, int lb, SB sb) {
    const float mA = j.invMassA, mB = j.invMassB, iA = j.invIA, iB = j.invIB;
    float2 vA = sb.v(la), vB = sb.v(lb);
    float wA = sb.w(la), wB = sb.w(lb);
    {                                                                   // spring
        float Cdot = (dot(j.ax, vB - vA) + j.sBx * wB) - j.sAx * wA;
        float impulse = -j.spring_mass * ((Cdot + j.bias) + j.gamma * j.impulse[1]);
        j.impulse[1] += impulse;
        float2 P = impulse * j.ax;
        float LA = impulse * j.sAx, LB = impulse * j.sBx;
        vA -= mA * P;
        wA -= iA * LA;
        vB += mB * P;
        wB += iB * LB;
    }
    {                                                                   // rotational motor
        float Cdot = (wB - wA) - j.motor_speed;
        float impulse = -j.motor_mass * Cdot;
        float oldImpulse = j.motor_impulse;
        float maxImpulse = x.dt * j.max_motor_torque;
        j.motor_impulse = bclamp(j.motor_impulse + impulse, -maxImpulse, maxImpulse);
        impulse = j.motor_impulse - oldImpulse;
        wA -= iA * impulse;
        wB += iB * impulse;
    }
    {                                                                   // point to line
        float Cdot = (dot(j.ay, vB - vA) + j.sBy * wB) - j.sAy * wA;
        float impulse = -j.mass[0] * Cdot;
        j.impulse[0] += impulse;
        float2 P = impulse * j.ay;
        float LA = impulse * j.sAy, LB = impulse * j.sBy;
        vA -= mA * P;
        wA -= iA * LA;
        vB += mB * P;
        wB += iB * LB;
    }
    sb.set_v(la, vA, wA);
    sb.set_v(lb, vB, wB);
}

__device__ __noinline__ bool wheel_solve_position(const DJoint& j, int la, int lb, SB sb) {
    float2 cA = sb.c(la), cB = sb.c(lb);
    float aA = sb.a(la), aB = sb.a(lb);
    Rot qA = rot(aA), qB = rot(aB);
    float2 rA = mul(qA, j.local_anchor_a - j.lcA);
    float2 rB = mul(qB, j.local_anchor_b - j.lcB);
    float2 d = ((cB - cA) + rB) - rA;
    float2 ay = mul(qA, j.local_axis_y);
    float sAy = cross(d + rA, ay);
    float sBy = cross(rB, ay);
    float C = dot(d, ay);
    // the effective mass uses the velocity pass's sAy / sBy, as the reference does
    float k = ((j.invMassA + j.invMassB) + (j.invIA * j.sAy) * j.sAy) + (j.invIB * j.sBy) * j.sBy;
    float impulse = k != 0.0f ? fdiv(-C, k) : 0.0f;
    float2 P = impulse * ay;
    float LA = impulse * sAy, LB = impulse * sBy;
    cA -= j.invMassA * P;
    aA -= j.invIA * LA;
    cB += j.invMassB * P;
    aB += j.invIB * LB;
    sb.set_c(la, cA, aA);
    sb.set_c(lb, cB, aB);
    return babs(C) <= kLinearSlop;
}

// ------------------------------------------------------------ prismatic joint (joints/b2prismaticjoint.d:391-757)
__device__ __noinline__ void prismatic_init(const Ctx& x, int ji, int b0, SB sb, bool warm, float dtRatio) {
    DJoint& j = x.jt[ji];
    const dbox_body_state& ba = x.bs[j.body_a];
    const dbox_body_state& bb = x.bs[j.body_b];
    int la = j.body_a - b0, lb = j.body_b - b0;
    j.lcA = b_lc(ba);
    j.lcB = b_lc(bb);
    j.invMassA = ba.mass[1];
    j.invMassB = bb.mass[1];
    j.invIA = ba.mass[3];
    j.invIB = bb.mass[3];
    float2 cA = sb.c(la), cB = sb.c(lb);
    float aA = sb.a(la), aB = sb.a(lb);
    float2 vA = sb.v(la), vB = sb.v(lb);
    float wA = sb.w(la), wB = sb.w(lb);
    Rot qA = rot(aA), qB = rot(aB);
    float2 rA = mul(qA, j.local_anchor_a - j.lcA);
    float2 rB = mul(qB, j.local_anchor_b - j.lcB);
    float2 d = ((cB - cA) + rB) - rA;
    const float mA = j.invMassA, mB = j.invMassB, iA = j.invIA, iB = j.invIB;
    j.axis = mul(qA, j.local_axis_x);                                   // motor
    j.a1 = cross(d + rA, j.axis);
    j.a2 = cross(rB, j.axis);
    float mm = ((mA + mB) + (iA * j.a1) * j.a1) + (iB * j.a2) * j.a2;
    if (mm > 0.0f) mm = fdiv(1.0f, mm);
    j.motor_mass = mm;
    j.perp = mul(qA, j.local_axis_y);                                   // prismatic constraint
    j.s1 = cross(d + rA, j.perp);
    j.s2 = cross(rB, j.perp);
    float k11 = ((mA + mB) + (iA * j.s1) * j.s1) + (iB * j.s2) * j.s2;
    float k12 = iA * j.s1 + iB * j.s2;
    float k13 = (iA * j.s1) * j.a1 + (iB * j.s2) * j.a2;
    float k22 = iA + iB;
    if (k22 == 0.0f) k22 = 1.0f;
    float k23 = iA * j.a1 + iB * j.a2;
    float k33 = ((mA + mB) + (iA * j.a1) * j.a1) + (iB * j.a2) * j.a2;
    j.mass[0] = k11; j.mass[1] = k12; j.mass[2] = k13;
    j.mass[3] = k12; j.mass[4] = k22; j.mass[5] = k23;
    j.mass[6] = k13; j.mass[7] = k23; j.mass[8] = k33;
    if (j.enable_limit) {
        float jointTranslation = dot(j.axis, d);
        if (babs(j.upper_translation - j.lower_translation) < 2.0f * kLinearSlop) {
            j.limit_state = 3;
        } else if (jointTranslation <= j.lower_translation) {
            if (j.limit_state != 1) { j.limit_state = 1; j.impulse[2] = 0.0f; }
        } else if (jointTranslation >= j.upper_translation) {
            if (j.limit_state != 2) { j.limit_state = 2; j.impulse[2] = 0.0f; }
        } else {
            j.limit_state = 0;
            j.impulse[2] = 0.0f;
        }
    } else {
        j.limit_state = 0;
        j.impulse[2] = 0.0f;
    }
    if (!j.enable_motor) j.motor_impulse = 0.0f;
    if (warm) {
        j.impulse[0] *= dtRatio; j.impulse[1] *= dtRatio; j.impulse[2] *= dtRatio;
        j.motor_impulse *= dtRatio;
        float2 P = j.impulse[0] * j.perp + (j.motor_impulse + j.impulse[2]) * j.axis;
        float LA = (j.impulse[0] * j.s1 + j.impulse[1]) + (j.motor_impulse + j.impulse[2]) * j.a1;
        float LB = (j.impulse[0] * j.s2 + j.impulse[1]) + (j.motor_impulse + j.impulse[2]) * j.a2;
        vA -= mA * P;
        wA -= iA * LA;
        vB += mB * P;
        wB += iB * LB;
    } else {
        j.impulse[0] = 0.0f; j.impulse[1] = 0.0f; j.impulse[2] = 0.0f;
        j.motor_impulse = 0.0f;
    }
    sb.set_v(la, vA, wA);
    sb.set_v(lb, vB, wB);
}

__device__ __noinline__ void prismatic_solve_velocity(const Ctx& x, DJoint& j, int la, int lb, SB sb) {
    float2 vA = sb.v(la), vB = sb.v(lb);
    float wA = sb.w(la), wB = sb.w(lb);
    const float mA = j.invMassA, mB = j.invMassB, iA = j.invIA, iB = j.invIB;
    if (j.enable_motor && j.limit_state != 3) {
        float Cdot = (dot(j.axis, vB - vA) + j.a2 * wB) - j.a1 * wA;
        float impulse = j.motor_mass * (j.motor_speed - Cdot);
        float oldImpulse = j.motor_impulse;
        float maxImpulse = x.dt * j.max_motor_force;
        j.motor_impulse = bclamp(j.motor_impulse + impulse, -maxImpulse, maxImpulse);
        impulse = j.motor_impulse - oldImpulse;
        float2 P = impulse * j.axis;
        float LA = impulse * j.a1, LB = impulse * j.a2;
        vA -= mA * P;
        wA -= iA * LA;
        vB += mB * P;
        wB += iB * LB;
    }
    float2 Cdot1;
    Cdot1.x = (dot(j.perp, vB - vA) + j.s2 * wB) - j.s1 * wA;
    Cdot1.y = wB - wA;
    if (j.enable_limit && j.limit_state != 0) {
        float Cdot2 = (dot(j.axis, vB - vA) + j.a2 * wB) - j.a1 * wA;
        float3 f1 = make_float3(j.impulse[0], j.impulse[1], j.impulse[2]);
        float3 df = solve33(j.mass, make_float3(-Cdot1.x, -Cdot1.y, -Cdot2));
        float3 imp = make_float3(f1.x + df.x, f1.y + df.y, f1.z + df.z);
        if (j.limit_state == 1) imp.z = bmax(imp.z, 0.0f);
        else if (j.limit_state == 2) imp.z = bmin(imp.z, 0.0f);
        float2 b = -Cdot1 - (imp.z - f1.z) * v2(j.mass[6], j.mass[7]);
        float2 f2r = solve22(j.mass, b) + v2(f1.x, f1.y);
        imp.x = f2r.x;
        imp.y = f2r.y;
        j.impulse[0] = imp.x; j.impulse[1] = imp.y; j.impulse[2] = imp.z;
        float3 d3 = make_float3(imp.x - f1.x, imp.y - f1.y, imp.z - f1.z);
        float2 P = d3.x * j.perp + d3.z * j.axis;
        float LA = (d3.x * j.s1 + d3.y) + d3.z * j.a1;
        float LB = (d3.x * j.s2 + d3.y) + d3.z * j.a2;
        vA -= mA * P;
        wA -= iA * LA;
        vB += mB * P;
        wB += iB * LB;
    } else {
        float2 df = solve22(j.mass, -Cdot1);
        j.impulse[0] += df.x;
        j.impulse[1] += df.y;
        float2 P = df.x * j.perp;
        float LA = df.x * j.s1 + df.y;
        float LB = df.x * j.s2 + df.y;
        vA -= mA * P;
        wA -= iA * LA;
        vB += mB * P;
        wB += iB * LB;
    }
    sb.set_v(la, vA, wA);
    sb.set_v(lb, vB, wB);
}

__device__ __noinline__ bool prismatic_solve_position(const DJoint& j, int la, int lb, SB sb) {
    float2 cA = sb.c(la), cB = sb.c(lb);
    float aA = sb.a(la), aB = sb.a(lb);
    Rot qA = rot(aA), qB = rot(aB);
    const float mA = j.invMassA, mB = j.invMassB, iA = j.invIA, iB = j.invIB;
    float2 rA = mul(qA, j.local_anchor_a - j.lcA);
    float2 rB = mul(qB, j.local_anchor_b - j.lcB);
    float2 d = ((cB + rB) - cA) - rA;
    float2 axis = mul(qA, j.local_axis_x);
    float a1 = cross(d + rA, axis);
    float a2 = cross(rB, axis);
    float2 perp = mul(qA, j.local_axis_y);
    float s1 = cross(d + rA, perp);
    float s2 = cross(rB, perp);
    float2 C1 = v2(dot(perp, d), (aB - aA) - j.reference_angle);
    float linearError = babs(C1.x);
    float angularError = babs(C1.y);
    bool active = false;
    float C2 = 0.0f;
    if (j.enable_limit) {
        float translation = dot(axis, d);
        if (babs(j.upper_translation - j.lower_translation) < 2.0f * kLinearSlop) {
            C2 = bclamp(translation, -kMaxLinearCorrection, kMaxLinearCorrection);
            linearError = bmax(linearError, babs(translation));
            active = true;
        } else if (translation <= j.lower_translation) {
            C2 = bclamp((translation - j.lower_translation) + kLinearSlop, -kMaxLinearCorrection, 0.0f);
            linearError = bmax(linearError, j.lower_translation - translation);
            active = true;
        } else if (translation >= j.upper_translation) {
            C2 = bclamp((translation - j.upper_translation) - kLinearSlop, 0.0f, kMaxLinearCorrection);
            linearError = bmax(linearError, translation - j.upper_translation);
            active = true;
        }
    }
    float3 imp;
    float k11 = ((mA + mB) + (iA * s1) * s1) + (iB * s2) * s2;
    float k12 = iA * s1 + iB * s2;
    float k22 = iA + iB;
    if (k22 == 0.0f) k22 = 1.0f;
    if (active) {
        float k13 = (iA * s1) * a1 + (iB * s2) * a2;
        float k23 = iA * a1 + iB * a2;
        float k33 = ((mA + mB) + (iA * a1) * a1) + (iB * a2) * a2;
        float K[9] = {k11, k12, k13, k12, k22, k23, k13, k23, k33};
        imp = solve33(K, make_float3(-C1.x, -C1.y, -C2));
    } else {
        float K[9] = {k11, k12, 0.0f, k12, k22, 0.0f, 0.0f, 0.0f, 0.0f};
        float2 i1 = solve22(K, -C1);
        imp = make_float3(i1.x, i1.y, 0.0f);
    }
    float2 P = imp.x * perp + imp.z * axis;
    float LA = (imp.x * s1 + imp.y) + imp.z * a1;
    float LB = (imp.x * s2 + imp.y) + imp.z * a2;
    cA -= mA * P;
    aA -= iA * LA;
    cB += mB * P;
    aB += iB * LB;
    sb.set_c(la, cA, aA);
    sb.set_c(lb, cB, aB);
    return linearError <= kLinearSlop && angularError <= kAngularSlop;
}

// ------------------------------------------------------------ pulley joint (joints/b2pulleyjoint.d:181-350)
__device__ __noinline__ void pulley_init(const Ctx& x, int ji, int b0, SB sb, bool warm, float dtRatio) {
    DJoint& j = x.jt[ji];
    const dbox_body_state& ba = x.bs[j.body_a];
    const dbox_body_state& bb = x.bs[j.body_b];
    int la = j.body_a - b0, lb = j.body_b - b0;
    j.lcA = b_lc(ba);
    j.lcB = b_lc(bb);
    j.invMassA = ba.mass[1];
    j.invMassB = bb.mass[1];
    j.invIA = ba.mass[3];
    j.invIB = bb.mass[3];
    float2 cA = sb.c(la), cB = sb.c(lb);
    float aA = sb.a(la), aB = sb.a(lb);
    float2 vA = sb.v(la), vB = sb.v(lb);
    float wA = sb.w(la), wB = sb.w(lb);
    Rot qA = rot(aA), qB = rot(aB);
    j.rA = mul(qA, j.local_anchor_a - j.lcA);
    j.rB = mul(qB, j.local_anchor_b - j.lcB);
    float2 uA = (cA + j.rA) - j.ground_a;
    float2 uB = (cB + j.rB) - j.ground_b;
    float lengthA = length(uA), lengthB = length(uB);
    if (lengthA > 10.0f * kLinearSlop) uA *= fdiv(1.0f, lengthA); else uA = v2(0.0f, 0.0f);
    if (lengthB > 10.0f * kLinearSlop) uB *= fdiv(1.0f, lengthB); else uB = v2(0.0f, 0.0f);
    j.uA = uA;
    j.uB = uB;
    float ruA = cross(j.rA, uA), ruB = cross(j.rB, uB);
    float mA = j.invMassA + (j.invIA * ruA) * ruA;
    float mB = j.invMassB + (j.invIB * ruB) * ruB;
    float mass = mA + (j.ratio * j.ratio) * mB;
    if (mass > 0.0f) mass = fdiv(1.0f, mass);
    j.mass[0] = mass;
    if (warm) {
        j.impulse[0] *= dtRatio;
        float2 PA = (-j.impulse[0]) * uA;
        float2 PB = ((-j.ratio) * j.impulse[0]) * uB;
        vA += j.invMassA * PA;
        wA += j.invIA * cross(j.rA, PA);
        vB += j.invMassB * PB;
        wB += j.invIB * cross(j.rB, PB);
    } else {
        j.impulse[0] = 0.0f;
    }
    sb.set_v(la, vA, wA);
    sb.set_v(lb, vB, wB);
}

__device__ __noinline__ void pulley_solve_velocity(DJoint& j, int la, int lb, SB sb) {
    float2 vA = sb.v(la), vB = sb.v(lb);
    float wA = sb.w(la), wB = sb.w(lb);
    float2 vpA = vA + cross(wA, j.rA);
    float2 vpB = vB + cross(wB, j.rB);
    float Cdot = (-dot(j.uA, vpA)) - j.ratio * dot(j.uB, vpB);
    float impulse = -j.mass[0] * Cdot;
    j.impulse[0] += impulse;
    float2 PA = (-impulse) * j.uA;
    float2 PB = ((-j.ratio) * impulse) * j.uB;
    vA += j.invMassA * PA;
    wA += j.invIA * cross(j.rA, PA);
    vB += j.invMassB * PB;
    wB += j.invIB * cross(j.rB, PB);
    sb.set_v(la, vA, wA);
    sb.set_v(lb, vB, wB);
}

__device__ __noinline__ bool pulley_solve_position(const DJoint& j, int la, int lb, SB sb) {
    float2 cA = sb.c(la), cB = sb.c(lb);
    float aA = sb.a(la), aB = sb.a(lb);
    Rot qA = rot(aA), qB = rot(aB);
    float2 rA = mul(qA, j.local_anchor_a - j.lcA);
    float2 rB = mul(qB, j.local_anchor_b - j.lcB);
    float2 uA = (cA + rA) - j.ground_a;
    float2 uB = (cB + rB) - j.ground_b;
    float lengthA = length(uA), lengthB = length(uB);
    if (lengthA > 10.0f * kLinearSlop) uA *= fdiv(1.0f, lengthA); else uA = v2(0.0f, 0.0f);
    if (lengthB > 10.0f * kLinearSlop) uB *= fdiv(1.0f, lengthB); else uB = v2(0.0f, 0.0f);
    float ruA = cross(rA, uA), ruB = cross(rB, uB);
    float mA = j.invMassA + (j.invIA * ruA) * ruA;
    float mB = j.invMassB + (j.invIB * ruB) * ruB;
    float mass = mA + (j.ratio * j.ratio) * mB;
    if (mass > 0.0f) mass = fdiv(1.0f, mass);
    float C = (j.constant - lengthA) - j.ratio * lengthB;
    float linearError = babs(C);
    float impulse = -mass * C;
    float2 PA = (-impulse) * uA;
    float2 PB = ((-j.ratio) * impulse) * uB;
    cA += j.invMassA * PA;
    aA += j.invIA * cross(rA, PA);
    cB += j.invMassB * PB;
    aB += j.invIB * cross(rB, PB);
    sb.set_c(la, cA, aA);
    sb.set_c(lb, cB, aB);
    return linearError < kLinearSlop;
}

// ------------------------------------------------------------ gear joint (joints/b2gearjoint.d:245-500)
// Four bodies: A (joint1's B), B (joint2's B), C (joint1's A), D (joint2's A); the level
// schedule gives the gear a level above the last constraint of each dynamic one.  Velocities
// and positions are written back A, B, C, D, as the reference does (C and D may coincide).
__device__ __noinline__ void gear_init(const Ctx& x, int ji, int b0, SB sb, bool warm) {
    DJoint& j = x.jt[ji];
    const dbox_body_state& bA = x.bs[j.body_a];
    const dbox_body_state& bB = x.bs[j.body_b];
    const dbox_body_state& bC = x.bs[j.body_c];
    const dbox_body_state& bD = x.bs[j.body_d];
    const int la = j.body_a - b0, lb = j.body_b - b0, lc = j.body_c - b0, ld = j.body_d - b0;
    j.lcA = b_lc(bA);
    j.lcB = b_lc(bB);
    j.lcC = b_lc(bC);
    j.lcD = b_lc(bD);
    j.invMassA = bA.mass[1];
    j.invMassB = bB.mass[1];
    j.invMassC = bC.mass[1];
    j.invMassD = bD.mass[1];
    j.invIA = bA.mass[3];
    j.invIB = bB.mass[3];
    j.invIC = bC.mass[3];
    j.invID = bD.mass[3];
    const float aA = sb.a(la), aB = sb.a(lb), aC = sb.a(lc), aD = sb.a(ld);
    float2 vA = sb.v(la), vB = sb.v(lb), vC = sb.v(lc), vD = sb.v(ld);
    float wA = sb.w(la), wB = sb.w(lb), wC = sb.w(lc), wD = sb.w(ld);
    const Rot qA = rot(aA), qB = rot(aB), qC = rot(aC), qD = rot(aD);
    float mass = 0.0f;
    if (j.type_a == kRevoluteJoint) {
        j.jv_ac = v2(0.0f, 0.0f);
        j.jw_a = 1.0f;
        j.jw_c = 1.0f;
        mass += j.invIA + j.invIC;
    } else {
        const float2 u = mul(qC, j.local_axis_c);
        const float2 rC = mul(qC, j.local_anchor_c - j.lcC);
        const float2 rA = mul(qA, j.local_anchor_a - j.lcA);
        j.jv_ac = u;
        j.jw_c = cross(rC, u);
        j.jw_a = cross(rA, u);
        mass += ((j.invMassC + j.invMassA) + (j.invIC * j.jw_c) * j.jw_c) + (j.invIA * j.jw_a) * j.jw_a;
    }
    if (j.type_b == kRevoluteJoint) {
        j.jv_bd = v2(0.0f, 0.0f);
        j.jw_b = j.ratio;
        j.jw_d = j.ratio;
        mass += (j.ratio * j.ratio) * (j.invIB + j.invID);
    } else {
        const float2 u = mul(qD, j.local_axis_d);
        const float2 rD = mul(qD, j.local_anchor_d - j.lcD);
        const float2 rB = mul(qB, j.local_anchor_b - j.lcB);
        j.jv_bd = j.ratio * u;
        j.jw_d = j.ratio * cross(rD, u);
        j.jw_b = j.ratio * cross(rB, u);
        mass += (((j.ratio * j.ratio) * (j.invMassD + j.invMassB)) + (j.invID * j.jw_d) * j.jw_d) + (j.invIB * j.jw_b) * j.jw_b;
    }
    j.mass[0] = mass > 0.0f ? fdiv(1.0f, mass) : 0.0f;
    if (warm) {                                                         // no dtRatio scaling here
        const float P = j.impulse[0];
        vA += (j.invMassA * P) * j.jv_ac;
        wA += (j.invIA * P) * j.jw_a;
        vB += (j.invMassB * P) * j.jv_bd;
        wB += (j.invIB * P) * j.jw_b;
        vC -= (j.invMassC * P) * j.jv_ac;
        wC -= (j.invIC * P) * j.jw_c;
        vD -= (j.invMassD * P) * j.jv_bd;
        wD -= (j.invID * P) * j.jw_d;
    } else {
        j.impulse[0] = 0.0f;
    }
    sb.set_v(la, vA, wA);
    sb.set_v(lb, vB, wB);
    sb.set_v(lc, vC, wC);
    sb.set_v(ld, vD, wD);
}

__device__ __noinline__ void gear_solve_velocity(DJoint& j, int b0, SB sb) {
    const int la = j.body_a - b0, lb = j.body_b - b0, lc = j.body_c - b0, ld = j.body_d - b0;
    float2 vA = sb.v(la), vB = sb.v(lb), vC = sb.v(lc), vD = sb.v(ld);
    float wA = sb.w(la), wB = sb.w(lb), wC = sb.w(lc), wD = sb.w(ld);
    float Cdot = dot(j.jv_ac, vA - vC) + dot(j.jv_bd, vB - vD);
    Cdot += ((j.jw_a * wA) - (j.jw_c * wC)) + ((j.jw_b * wB) - (j.jw_d * wD));
    const float impulse = (-j.mass[0]) * Cdot;
    j.impulse[0] += impulse;
    vA += (j.invMassA * impulse) * j.jv_ac;
    wA += (j.invIA * impulse) * j.jw_a;
    vB += (j.invMassB * impulse) * j.jv_bd;
    wB += (j.invIB * impulse) * j.jw_b;
    vC -= (j.invMassC * impulse) * j.jv_ac;
    wC -= (j.invIC * impulse) * j.jw_c;
    vD -= (j.invMassD * impulse) * j.jv_bd;
    wD -= (j.invID * impulse) * j.jw_d;
    sb.set_v(la, vA, wA);
    sb.set_v(lb, vB, wB);
    sb.set_v(lc, vC, wC);
    sb.set_v(ld, vD, wD);
}

__device__ __noinline__ bool gear_solve_position(const DJoint& j, int b0, SB sb) {
    const int la = j.body_a - b0, lb = j.body_b - b0, lc = j.body_c - b0, ld = j.body_d - b0;
    float2 cA = sb.c(la), cB = sb.c(lb), cC = sb.c(lc), cD = sb.c(ld);
    float aA = sb.a(la), aB = sb.a(lb), aC = sb.a(lc), aD = sb.a(ld);
    const Rot qA = rot(aA), qB = rot(aB), qC = rot(aC), qD = rot(aD);
    float coordinateA = 0.0f, coordinateB = 0.0f;
    float2 JvAC = v2(0.0f, 0.0f), JvBD = v2(0.0f, 0.0f);
    float JwA = 0.0f, JwB = 0.0f, JwC = 0.0f, JwD = 0.0f;
    float mass = 0.0f;
    if (j.type_a == kRevoluteJoint) {
        JwA = 1.0f;
        JwC = 1.0f;
        mass += j.invIA + j.invIC;
        coordinateA = (aA - aC) - j.reference_angle_a;
    } else {
        const float2 u = mul(qC, j.local_axis_c);
        const float2 rC = mul(qC, j.local_anchor_c - j.lcC);
        const float2 rA = mul(qA, j.local_anchor_a - j.lcA);
        JvAC = u;
        JwC = cross(rC, u);
        JwA = cross(rA, u);
        mass += ((j.invMassC + j.invMassA) + (j.invIC * JwC) * JwC) + (j.invIA * JwA) * JwA;
        const float2 pC = j.local_anchor_c - j.lcC;
        const float2 pA = mulT(qC, rA + (cA - cC));
        coordinateA = dot(pA - pC, j.local_axis_c);
    }
    if (j.type_b == kRevoluteJoint) {
        JwB = j.ratio;
        JwD = j.ratio;
        mass += (j.ratio * j.ratio) * (j.invIB + j.invID);
        coordinateB = (aB - aD) - j.reference_angle_b;
    } else {
        const float2 u = mul(qD, j.local_axis_d);
        const float2 rD = mul(qD, j.local_anchor_d - j.lcD);
        const float2 rB = mul(qB, j.local_anchor_b - j.lcB);
        JvBD = j.ratio * u;
        JwD = j.ratio * cross(rD, u);
        JwB = j.ratio * cross(rB, u);
        mass += (((j.ratio * j.ratio) * (j.invMassD + j.invMassB)) + (j.invID * JwD) * JwD) + (j.invIB * JwB) * JwB;
        const float2 pD = j.local_anchor_d - j.lcD;
        const float2 pB = mulT(qD, rB + (cB - cD));
        coordinateB = dot(pB - pD, j.local_axis_d);
    }
    const float C = (coordinateA + j.ratio * coordinateB) - j.constant;
    float impulse = 0.0f;
    if (mass > 0.0f) impulse = fdiv(-C, mass);
    cA += (j.invMassA * impulse) * JvAC;
    aA += (j.invIA * impulse) * JwA;
    cB += (j.invMassB * impulse) * JvBD;
    aB += (j.invIB * impulse) * JwB;
    cC -= (j.invMassC * impulse) * JvAC;
    aC -= (j.invIC * impulse) * JwC;
    cD -= (j.invMassD * impulse) * JvBD;
    aD -= (j.invID * impulse) * JwD;
    sb.set_c(la, cA, aA);
    sb.set_c(lb, cB, aB);
    sb.set_c(lc, cC, aC);
    sb.set_c(ld, cD, aD);
    return true;                                                        // linearError stays 0
}

// ------------------------------------------------------------ mouse joint (joints/b2mousejoint.d:132-226), body B only
__device__ __noinline__ void mouse_init(const Ctx& x, int ji, int b0, SB sb, bool warm, float dtRatio) {
    DJoint& j = x.jt[ji];
    const dbox_body_state& bb = x.bs[j.body_b];
    int lb = j.body_b - b0;
    j.lcB = b_lc(bb);
    j.invMassB = bb.mass[1];
    j.invIB = bb.mass[3];
    float2 cB = sb.c(lb);
    float aB = sb.a(lb);
    float2 vB = sb.v(lb);
    float wB = sb.w(lb);
    Rot qB = rot(aB);
    float mass = bb.mass[0];
    float omega = (2.0f * kPi) * j.frequency_hz;
    float d = ((2.0f * mass) * j.damping_ratio) * omega;
    float k = mass * (omega * omega);
    float h = x.dt;
    float gamma = h * (d + h * k);
    if (gamma != 0.0f) gamma = fdiv(1.0f, gamma);
    j.gamma = gamma;
    j.beta = (h * k) * gamma;
    j.rB = mul(qB, j.local_anchor_b - j.lcB);
    float k11 = (j.invMassB + (j.invIB * j.rB.y) * j.rB.y) + gamma;
    float k21 = ((-j.invIB) * j.rB.x) * j.rB.y;
    float k22 = (j.invMassB + (j.invIB * j.rB.x) * j.rB.x) + gamma;
    float det = k11 * k22 - k21 * k21;                                  // b2Mat22.GetInverse
    if (det != 0.0f) det = fdiv(1.0f, det);
    j.mass[0] = det * k22;
    j.mass[3] = -det * k21;
    j.mass[1] = -det * k21;
    j.mass[4] = det * k11;
    float2 C = (cB + j.rB) - j.target;
    C *= j.beta;
    j.mouse_c = C;
    wB *= 0.98f;                                                        // the reference's extra damping
    if (warm) {
        j.impulse[0] *= dtRatio;
        j.impulse[1] *= dtRatio;
        float2 I = v2(j.impulse[0], j.impulse[1]);
        vB += j.invMassB * I;
        wB += j.invIB * cross(j.rB, I);
    } else {
        j.impulse[0] = 0.0f;
        j.impulse[1] = 0.0f;
    }
    sb.set_v(lb, vB, wB);
}

__device__ __noinline__ void mouse_solve_velocity(const Ctx& x, DJoint& j, int lb, SB sb) {
    float2 vB = sb.v(lb);
    float wB = sb.w(lb);
    float2 Cdot = vB + cross(wB, j.rB);
    float2 I = v2(j.impulse[0], j.impulse[1]);
    float2 rhs = -((Cdot + j.mouse_c) + j.gamma * I);
    float2 impulse = v2(j.mass[0] * rhs.x + j.mass[3] * rhs.y, j.mass[1] * rhs.x + j.mass[4] * rhs.y);
    float2 oldImpulse = I;
    I += impulse;
    float maxImpulse = x.dt * j.max_force;
    if (I.x * I.x + I.y * I.y > maxImpulse * maxImpulse) I *= fdiv(maxImpulse, length(I));
    j.impulse[0] = I.x;
    j.impulse[1] = I.y;
    impulse = I - oldImpulse;
    vB += j.invMassB * impulse;
    wB += j.invIB * cross(j.rB, impulse);
    sb.set_v(lb, vB, wB);
}

// ------------------------------------------------------------ revolute joint (joints/b2revolutejoint.d:319-636)
DG void joint_init(const Ctx& x, int ji, int b0, SB sb, bool warm, float dtRatio) {
    switch (x.jt[ji].type) {
    case kDistanceJoint: distance_init(x, ji, b0, sb, warm, dtRatio); return;
    case kRopeJoint: rope_init(x, ji, b0, sb, warm, dtRatio); return;
    case kWeldJoint: weld_init(x, ji, b0, sb, warm, dtRatio); return;
    case kFrictionJoint:
    case kMotorJoint: friction_motor_init(x, ji, b0, sb, warm, dtRatio); return;
    case kWheelJoint: wheel_init(x, ji, b0, sb, warm, dtRatio); return;
    case kPrismaticJoint: prismatic_init(x, ji, b0, sb, warm, dtRatio); return;
    case kPulleyJoint: pulley_init(x, ji, b0, sb, warm, dtRatio); return;
    case kMouseJoint: mouse_init(x, ji, b0, sb, warm, dtRatio); return;
    case kGearJoint: gear_init(x, ji, b0, sb, warm); return;
    default: break;
    }
    DJoint& j = x.jt[ji];
    const dbox_body_state& ba = x.bs[j.body_a];
    const dbox_body_state& bb = x.bs[j.body_b];
    int la = j.body_a - b0, lb = j.body_b - b0;
    j.lcA = b_lc(ba);
    j.lcB = b_lc(bb);
    j.invMassA = ba.mass[1];
    j.invMassB = bb.mass[1];
    j.invIA = ba.mass[3];
    j.invIB = bb.mass[3];
    float aA = sb.a(la);
    float2 vA = sb.v(la);
    float wA = sb.w(la);
    float aB = sb.a(lb);
    float2 vB = sb.v(lb);
    float wB = sb.w(lb);
    Rot qA = rot(aA), qB = rot(aB);
    j.rA = mul(qA, j.local_anchor_a - j.lcA);
    j.rB = mul(qB, j.local_anchor_b - j.lcB);
    float mA = j.invMassA, mB = j.invMassB, iA = j.invIA, iB = j.invIB;
    bool fixedRotation = (iA + iB == 0.0f);
    float2 rA = j.rA, rB = j.rB;
    j.mass[0] = ((mA + mB) + (rA.y * rA.y) * iA) + (rB.y * rB.y) * iB;   // ex.x
    j.mass[3] = (-rA.y * rA.x) * iA - (rB.y * rB.x) * iB;               // ey.x
    j.mass[6] = -rA.y * iA - rB.y * iB;                                  // ez.x
    j.mass[1] = j.mass[3];                                               // ex.y
    j.mass[4] = ((mA + mB) + (rA.x * rA.x) * iA) + (rB.x * rB.x) * iB;   // ey.y
    j.mass[7] = rA.x * iA + rB.x * iB;                                   // ez.y
    j.mass[2] = j.mass[6];                                               // ex.z
    j.mass[5] = j.mass[7];                                               // ey.z
    j.mass[8] = iA + iB;                                                 // ez.z
    j.motor_mass = iA + iB;
    if (j.motor_mass > 0.0f) j.motor_mass = fdiv(1.0f, j.motor_mass);
    if (j.enable_motor == 0 || fixedRotation) j.motor_impulse = 0.0f;
    if (j.enable_limit && !fixedRotation) {
        float jointAngle = (aB - aA) - j.reference_angle;
        if (babs(j.upper_angle - j.lower_angle) < 2.0f * kAngularSlop) {
            j.limit_state = 3;
        } else if (jointAngle <= j.lower_angle) {
            if (j.limit_state != 1) j.impulse[2] = 0.0f;
            j.limit_state = 1;
        } else if (jointAngle >= j.upper_angle) {
            if (j.limit_state != 2) j.impulse[2] = 0.0f;
            j.limit_state = 2;
        } else {
            j.limit_state = 0;
            j.impulse[2] = 0.0f;
        }
    } else {
        j.limit_state = 0;
    }
    if (warm) {
        j.impulse[0] *= dtRatio; j.impulse[1] *= dtRatio; j.impulse[2] *= dtRatio;
        j.motor_impulse *= dtRatio;
        float2 P = v2(j.impulse[0], j.impulse[1]);
        vA -= mA * P;
        wA -= iA * ((cross(rA, P) + j.motor_impulse) + j.impulse[2]);
        vB += mB * P;
        wB += iB * ((cross(rB, P) + j.motor_impulse) + j.impulse[2]);
    } else {
        j.impulse[0] = j.impulse[1] = j.impulse[2] = 0.0f;
        j.motor_impulse = 0.0f;
    }
    sb.set_v(la, vA, wA);
    sb.set_v(lb, vB, wB);
}

DG void joint_solve_velocity(const Ctx& x, int ji, int b0, SB sb) {
    DJoint& j = x.jt[ji];
    int la = j.body_a - b0, lb = j.body_b - b0;
    if (j.type == kDistanceJoint) { distance_solve_velocity(j, la, lb, sb); return; }
    if (j.type == kRopeJoint) { rope_solve_velocity(x, j, la, lb, sb); return; }
    if (j.type == kWeldJoint) { weld_solve_velocity(j, la, lb, sb); return; }
    if (j.type == kFrictionJoint || j.type == kMotorJoint) { friction_motor_solve_velocity(x, j, la, lb, sb); return; }
    if (j.type == kWheelJoint) { wheel_solve_velocity(x, j, la, lb, sb); return; }
    if (j.type == kPrismaticJoint) { prismatic_solve_velocity(x, j, la, lb, sb); return; }
    if (j.type == kPulleyJoint) { pulley_solve_velocity(j, la, lb, sb); return; }
    if (j.type == kMouseJoint) { mouse_solve_velocity(x, j, lb, sb); return; }
    if (j.type == kGearJoint) { gear_solve_velocity(j, b0, sb); return; }
    float2 vA = sb.v(la), vB = sb.v(lb);
    float wA = sb.w(la), wB = sb.w(lb);
    float mA = j.invMassA, mB = j.invMassB, iA = j.invIA, iB = j.invIB;
    bool fixedRotation = (iA + iB == 0.0f);
    if (j.enable_motor && j.limit_state != 3 && !fixedRotation) {
        float Cdot = (wB - wA) - j.motor_speed;
        float imp = -j.motor_mass * Cdot;
        float oldImpulse = j.motor_impulse;
        float maxImpulse = x.dt * j.max_motor_torque;
        j.motor_impulse = bclamp(j.motor_impulse + imp, -maxImpulse, maxImpulse);
        imp = j.motor_impulse - oldImpulse;
        wA -= iA * imp;
        wB += iB * imp;
    }
    if (j.enable_limit && j.limit_state != 0 && !fixedRotation) {
        float2 Cdot1 = ((vB + cross(wB, j.rB)) - vA) - cross(wA, j.rA);
        float Cdot2 = wB - wA;
        float3 r = solve33(j.mass, make_float3(Cdot1.x, Cdot1.y, Cdot2));
        float3 imp = make_float3(-r.x, -r.y, -r.z);
        if (j.limit_state == 3) {
            j.impulse[0] += imp.x; j.impulse[1] += imp.y; j.impulse[2] += imp.z;
        } else if (j.limit_state == 1 || j.limit_state == 2) {
            float newImpulse = j.impulse[2] + imp.z;
            bool reduce = j.limit_state == 1 ? newImpulse < 0.0f : newImpulse > 0.0f;
            if (reduce) {
                float2 rhs = -Cdot1 + j.impulse[2] * v2(j.mass[6], j.mass[7]);
                float2 reduced = solve22(j.mass, rhs);
                imp.x = reduced.x;
                imp.y = reduced.y;
                imp.z = -j.impulse[2];
                j.impulse[0] += reduced.x;
                j.impulse[1] += reduced.y;
                j.impulse[2] = 0.0f;
            } else {
                j.impulse[0] += imp.x; j.impulse[1] += imp.y; j.impulse[2] += imp.z;
            }
        }
        float2 P = v2(imp.x, imp.y);
        vA -= mA * P;
        wA -= iA * (cross(j.rA, P) + imp.z);
        vB += mB * P;
        wB += iB * (cross(j.rB, P) + imp.z);
    } else {
        float2 Cdot = ((vB + cross(wB, j.rB)) - vA) - cross(wA, j.rA);
        float2 imp = solve22(j.mass, -Cdot);
        j.impulse[0] += imp.x;
        j.impulse[1] += imp.y;
        vA -= mA * imp;
        wA -= iA * cross(j.rA, imp);
        vB += mB * imp;
        wB += iB * cross(j.rB, imp);
    }
    sb.set_v(la, vA, wA);
    sb.set_v(lb, vB, wB);
}

DG bool joint_solve_position(const Ctx& x, int ji, int b0, SB sb) {
    DJoint& j = x.jt[ji];
    int la = j.body_a - b0, lb = j.body_b - b0;
    if (j.type == kDistanceJoint) return distance_solve_position(j, la, lb, sb);
    if (j.type == kRopeJoint) return rope_solve_position(j, la, lb, sb);
    if (j.type == kWeldJoint) return weld_solve_position(j, la, lb, sb);
    if (j.type == kFrictionJoint || j.type == kMotorJoint) return true;   // no position correction
    if (j.type == kWheelJoint) return wheel_solve_position(j, la, lb, sb);
    if (j.type == kPrismaticJoint) return prismatic_solve_position(j, la, lb, sb);
    if (j.type == kPulleyJoint) return pulley_solve_position(j, la, lb, sb);
    if (j.type == kMouseJoint) return true;
    if (j.type == kGearJoint) return gear_solve_position(j, b0, sb);
    float2 cA = sb.c(la), cB = sb.c(lb);
    float aA = sb.a(la), aB = sb.a(lb);
    float angularError = 0.0f, positionError = 0.0f;
    bool fixedRotation = (j.invIA + j.invIB == 0.0f);
    if (j.enable_limit && j.limit_state != 0 && !fixedRotation) {
        float angle = (aB - aA) - j.reference_angle;
        float limitImpulse = 0.0f;
        if (j.limit_state == 3) {
            float C = bclamp(angle - j.lower_angle, -kMaxAngularCorrection, kMaxAngularCorrection);
            limitImpulse = -j.motor_mass * C;
            angularError = babs(C);
        } else if (j.limit_state == 1) {
            float C = angle - j.lower_angle;
            angularError = -C;
            C = bclamp(C + kAngularSlop, -kMaxAngularCorrection, 0.0f);
            limitImpulse = -j.motor_mass * C;
        } else if (j.limit_state == 2) {
            float C = angle - j.upper_angle;
            angularError = C;
            C = bclamp(C - kAngularSlop, 0.0f, kMaxAngularCorrection);
            limitImpulse = -j.motor_mass * C;
        }
        aA -= j.invIA * limitImpulse;
        aB += j.invIB * limitImpulse;
    }
    {
        Rot qA = rot(aA), qB = rot(aB);
        float2 rA = mul(qA, j.local_anchor_a - j.lcA);
        float2 rB = mul(qB, j.local_anchor_b - j.lcB);
        float2 C = ((cB + rB) - cA) - rA;
        positionError = length(C);
        float mA = j.invMassA, mB = j.invMassB, iA = j.invIA, iB = j.invIB;
        float K[9];
        K[0] = ((mA + mB) + (iA * rA.y) * rA.y) + (iB * rB.y) * rB.y;     // ex.x
        K[1] = ((-iA * rA.x) * rA.y) - (iB * rB.x) * rB.y;               // ex.y
        K[3] = K[1];                                                      // ey.x
        K[4] = ((mA + mB) + (iA * rA.x) * rA.x) + (iB * rB.x) * rB.x;     // ey.y
        float2 s = solve22(K, C);
        float2 imp = -s;
        cA -= mA * imp;
        aA -= iA * cross(rA, imp);
        cB += mB * imp;
        aB += iB * cross(rB, imp);
    }
    sb.set_c(la, cA, aA);
    sb.set_c(lb, cB, aB);
    return positionError <= kLinearSlop && angularError <= kAngularSlop;
}

// ------------------------------------------------------------ level schedule
// Items: contact slot c >= 0, joint j encoded as -(j + 1).  Bodies are world-local.
DG void item_bodies(const Ctx& x, int item, int b0, int& A, int& B) {
    if (item >= 0) { int2 cb = x.s_cbody[item]; A = cb.x; B = cb.y; }
    else { const DJoint& j = x.jt[-item - 1]; A = j.body_a - b0; B = j.body_b - b0; }
}

// Build one level schedule for world w (all lanes).  `contacts_first` gives the warm-start /
// position order of b2Island.Solve (contacts then joints, b2island.d:136-146 and 206-224);
// otherwise the velocity-iteration order (joints then contacts, b2island.d:153-161).
// Lane 0 walks the island sequence once and gives each constraint the level 1 + the last
// level of its dynamic bodies; the warp then buckets the constraints by level.  Level L
// items end up in sched[kx + lvl[kx+L] .. kx + lvl[kx+L+1]) (in any order inside a level:
// they share no dynamic body).  Returns the number of levels.
DG int build_schedule(const Ctx& x, const WorldInfo& wi, int nIsl, bool contacts_first, const unsigned char* vbf,
                      int* last, int* sched, int* lvl) {
    const int b0 = wi.body_start, kx = wi.kx_start, c0 = wi.contact_start;
    const int lane = lane_id();
    for (int i = lane; i < wi.body_count; i += kWarp) last[i] = 0;
    tsync();
    int maxL = 0, n = 0;
    // islands share no dynamic body, so the levels are the same whether each island's
    // constraints are walked island by island or all contacts (in island order) are walked
    // before all joints (or after, for the velocity order): no per-island loop is needed.
    // 32 constraints at a time: each lane loads one constraint's bodies and their dynamic
    // flags, then the warp walks the 32 in order with the bodies passed by shuffles (the
    // walk's only carried state is `last`, read by every lane and written by lane 0)
    const int ncT = x.s_isl_cstart[wi.bx_start + nIsl], njT = x.s_isl_jstart[wi.bx_start + nIsl];
    for (int pass = 0; pass < 2; ++pass) {
        const bool doContacts = (pass == 0) == contacts_first;
        const int e = doContacts ? ncT : njT;
        for (int base = 0; base < e; base += kWarp) {
            const int t = base + lane;
            int item = 0, A = 0, B = 0, C = 0, D = 0;
            unsigned dm = 0;                           // dynamic A, B, C, D in bits 0..3
            if (t < e) {
                if (doContacts) {
                    item = x.s_isl_contact[c0 + t];
                    const int2 pr = x.s_isl_pair[c0 + t];
                    A = pr.x;
                    B = pr.y;
                } else {
                    item = -(x.s_isl_joint[wi.joint_start + t] + 1);
                    item_bodies(x, item, b0, A, B);
                    const DJoint& jj = x.jt[-item - 1];
                    if (jj.type == kGearJoint) {                    // a gear also moves C and D
                        C = jj.body_c - b0;
                        D = jj.body_d - b0;
                        dm |= ((vbf[C] & kBfDynamic) ? 4u : 0u) | ((vbf[D] & kBfDynamic) ? 8u : 0u);
                    }
                }
                dm |= ((vbf[A] & kBfDynamic) ? 1u : 0u) | ((vbf[B] & kBfDynamic) ? 2u : 0u);
            }
            const int cnt = e - base < kWarp ? e - base : kWarp;
            int myl = 0;
            for (int j = 0; j < cnt; ++j) {
                const int a = __shfl_sync(0xffffffffu, A, j), bb = __shfl_sync(0xffffffffu, B, j);
                const int c = __shfl_sync(0xffffffffu, C, j), d = __shfl_sync(0xffffffffu, D, j);
                const unsigned m = __shfl_sync(0xffffffffu, dm, j);
                int la = (m & 1u) ? last[a] : 0, lb = (m & 2u) ? last[bb] : 0;
                int l = (la > lb ? la : lb);
                if ((m & 4u) && last[c] > l) l = last[c];
                if ((m & 8u) && last[d] > l) l = last[d];
                l += 1;
                __syncwarp();
                if (lane == 0) {
                    if (m & 1u) last[a] = l;
                    if (m & 2u) last[bb] = l;
                    if (m & 4u) last[c] = l;
                    if (m & 8u) last[d] = l;
                }
                __syncwarp();
                if (lane == j) myl = l;
                if (l > maxL) maxL = l;
            }
            if (t < e) {
                x.s_level[kx + n + lane] = myl;
                x.s_tmp[kx + n + lane] = item;
            }
            n += cnt;
        }
    }
    maxL = __shfl_sync(0xffffffffu, maxL, 0);
    n = __shfl_sync(0xffffffffu, n, 0);
    for (int l = lane; l <= maxL + 1; l += kWarp) lvl[kx + l] = 0;
    tsync();
    for (int i = lane; i < n; i += kWarp) atomicAdd(&lvl[kx + x.s_level[kx + i]], 1);
    tsync();
    int total = 0;
    for (int base = 0; base <= maxL + 1; base += kWarp) {
        int l = base + lane;
        int v = l <= maxL + 1 ? lvl[kx + l] : 0;
        int incl = v;
        for (int o = 1; o < 32; o <<= 1) {
            int t = __shfl_up_sync(0xffffffffu, incl, o);
            if (lane >= o) incl += t;
        }
        if (l <= maxL + 1) {
            lvl[kx + l] = total + incl - v;
            x.s_lcur[kx + l] = total + incl - v;
        }
        total += __shfl_sync(0xffffffffu, incl, 31);
    }
    tsync();
    for (int i = lane; i < n; i += kWarp) {
        int pos = atomicAdd(&x.s_lcur[kx + x.s_level[kx + i]], 1);
        sched[kx + pos] = x.s_tmp[kx + i];
    }
    tsync();
    return maxL;
}

// island id of a constraint: the island of one of its non-static bodies
DG int item_island(const Ctx& x, int item, int b0) {
    int A, B;
    item_bodies(x, item, b0, A, B);
    return (x.s_bfl[b0 + A] & kBfStatic) ? x.s_body_island[b0 + B] : x.s_body_island[b0 + A];
}

// b2Fixture.Synchronize + b2DynamicTree.MoveProxy for every fixture of body b
// (b2body.d:1129-1141, b2fixture.d:480-502, b2dynamictree.d:140-184)
DG void sync_fixtures(const Ctx& x, int b) {
    const dbox_body_state& B = x.bs[b];
    Xf xf1;
    xf1.q = rot(B.sweep[6]);
    xf1.p = v2(B.sweep[2], B.sweep[3]) - mul(xf1.q, b_lc(B));
    Xf xf2 = b_xf(B);
    const BodyStatic& st = x.bst[b];
    for (int e = 0; e < st.fix_count; ++e) {
        int f = x.body_fix[st.fix_start + e];
        dbox_proxy_state& p = x.px[f];
        if (p.proxy_id < 0) continue;
        AABB a1 = fixture_aabb(x.fx[f], xf1);
        AABB a2 = fixture_aabb(x.fx[f], xf2);
        AABB aabb;
        aabb.lo = vmin(a1.lo, a2.lo);
        aabb.hi = vmax(a1.hi, a2.hi);
        float2 displacement = xf2.p - xf1.p;
        AABB fat = proxy_fat(x, f);
        if (aabb_contains(fat, aabb)) continue;
        float2 r = v2(kAabbExtension, kAabbExtension);
        aabb.lo = aabb.lo - r;
        aabb.hi = aabb.hi + r;
        float2 d = kAabbMultiplier * displacement;
        if (d.x < 0.0f) aabb.lo.x += d.x; else aabb.hi.x += d.x;
        if (d.y < 0.0f) aabb.lo.y += d.y; else aabb.hi.y += d.y;
        p.fat_aabb[0] = aabb.lo.x; p.fat_aabb[1] = aabb.lo.y;
        p.fat_aabb[2] = aabb.hi.x; p.fat_aabb[3] = aabb.hi.y;
        p.moved = 1;
    }
}

// per-contact compact data for the sequential walks: world-local bodies, and
// s_cq bit0 = enabled & touching & no sensor (island graph edge), bit1 = a sensor fixture
DG void contact_compact(const Ctx& x, int ci, int b0) {
    const dbox_contact_state& c = x.ct[ci];
    const DFixture& fa = x.fx[c.fixture_a];
    const DFixture& fb = x.fx[c.fixture_b];
    x.s_cbody[ci] = make_int2(fa.body - b0, fb.body - b0);
    int sensor = (fa.sensor || fb.sensor) ? 1 : 0;
    int edge = ((c.flags & kContactEnabled) && (c.flags & kContactTouching) && !sensor) ? 1 : 0;
    x.s_cq[ci] = (unsigned char)(edge | (sensor << 1));
}

DG unsigned char body_flag_byte(const dbox_body_state& b) {
    unsigned char f = 0;
    if (b.flags & kBodyAwake) f |= kBfAwake;
    if (b.flags & kBodyActive) f |= kBfActive;
    if (b.type == kStaticBody) f |= kBfStatic;
    if (b.type == kDynamicBody) f |= kBfDynamic;
    return f;
}

// Learned start, first velocity iteration (b2contactsolver.d:492-772 run twice): the contact
// is solved from its predicted start and from the zero start of its new points (the
// prediction's warm-start impulse taken back out of the two bodies), each on a private copy
// of the two bodies' velocities; the start whose first correction |dlambda| is smaller
// wins (the prediction on ties) and its velocities and impulses are kept.
__device__ __noinline__ void solve_velocity_learned(const VRow& r, SB sb, float4* imp) {
    VC vp = unpack_v(r);
    const int ids = r.ids.z;
    VC vz = vp;
    float2 vA = sb.v(vp.bodyA), vB = sb.v(vp.bodyB);
    float wA = sb.w(vp.bodyA), wB = sb.w(vp.bodyB);
    float2 vA0 = vA, vB0 = vB;
    float wA0 = wA, wB0 = wB;
    float2 n = vp.normal, t = cross(n, 1.0f);
    for (int j = 0; j < 2; ++j) {
        if (!(ids & (0x200 << j)) || j >= vp.pointCount) continue;
        float2 P = vp.p[j].normalImpulse * n + vp.p[j].tangentImpulse * t;
        vA0 += vp.invMassA * P;
        wA0 += vp.invIA * cross(vp.p[j].rA, P);
        vB0 -= vp.invMassB * P;
        wB0 -= vp.invIB * cross(vp.p[j].rB, P);
        vz.p[j].normalImpulse = 0.0f;
        vz.p[j].tangentImpulse = 0.0f;
    }
    float la[12] = {vA.x, vA.y, wA, 0.0f, 0.0f, 0.0f, vB.x, vB.y, wB, 0.0f, 0.0f, 0.0f};
    float lz[12] = {vA0.x, vA0.y, wA0, 0.0f, 0.0f, 0.0f, vB0.x, vB0.y, wB0, 0.0f, 0.0f, 0.0f};
    SB sa, sz;
    sa.p = la;
    sz.p = lz;
    VC pa = vp, pz = vz;
    pa.bodyA = 0; pa.bodyB = 1;
    pz.bodyA = 0; pz.bodyB = 1;
    solve_velocity(pa, sa);
    solve_velocity(pz, sz);
    float ra = 0.0f, rz = 0.0f;
    for (int j = 0; j < vp.pointCount; ++j) {
        float dn = pa.p[j].normalImpulse - vp.p[j].normalImpulse, dt = pa.p[j].tangentImpulse - vp.p[j].tangentImpulse;
        ra += dn * dn + dt * dt;
        dn = pz.p[j].normalImpulse - vz.p[j].normalImpulse;
        dt = pz.p[j].tangentImpulse - vz.p[j].tangentImpulse;
        rz += dn * dn + dt * dt;
    }
    const bool zero = rz < ra;
    const float* st = zero ? lz : la;
    const VC& ch = zero ? pz : pa;
    sb.set_v(vp.bodyA, v2(st[0], st[1]), st[2]);
    sb.set_v(vp.bodyB, v2(st[6], st[7]), st[8]);
    *imp = make_float4(ch.p[0].normalImpulse, ch.p[0].tangentImpulse, ch.p[1].normalImpulse, ch.p[1].tangentImpulse);
}

// The warm-start modes' part of a contact row (modes 1..3, b2contactsolver.d:244-450 itself
// unchanged): the points whose impulse started from zero (no feature-id match in Collide) are
// marked in the row; mode 1 logs the contact's features as a training sample (its targets
// follow at StoreImpulses), mode 2 stores them for a prediction, mode 3 sets those points to
// the given start.  Returns whether the row waits for a prediction.
DG bool row_start_modes(const Ctx& x, int item, int slog_at, const VC& vc, const PC& pc, const float* sep, SB sb,
                        float h, VRow& vr) {
    unsigned fr = x.ct[item].flags & (kContactNew0 | kContactNew1);
    if (pc.pointCount < 2) fr &= ~(unsigned)kContactNew1;
    if (x.ws_mode == 1) x.s_slog[slog_at] = -1;
    if (!fr) return false;
    vr.ids.z |= (fr & kContactNew0 ? 0x200 : 0) | (fr & kContactNew1 ? 0x400 : 0);
    float* f = x.ws_mode == 1 ? nullptr : x.s_feat + (size_t)kFeat * item;
    if (x.ws_mode == 1) {
        unsigned slot = atomicAdd(x.sample_count, 1u);
        if ((int)slot < x.sample_cap) {
            f = x.samples + (size_t)kSampleFloats * slot;
            x.s_slog[slog_at] = (int)slot;
        }
    }
    if (f) {
        float fv[kFeat];
        contact_features(vc, sep, pc.pointCount, sb, x.gravity, h, fv);
#pragma unroll
        for (int q = 0; q < kFeat; ++q) f[q] = fv[q];
    }
    if (x.ws_mode == 3 && x.start_ct) {
        // given start: the impulses another handle's step from the same state ended with at
        // this contact slot (clamped as a prediction is), from the point with the same feature
        // id (the source's SolveTOI may have re-evaluated the manifold after its solve)
        const dbox_contact_state& g = x.start_ct[item];
        for (int j = 0; j < pc.pointCount; ++j) {
            if (!(fr & (j == 0 ? kContactNew0 : kContactNew1))) continue;
            const uint32_t id = x.ct[item].points[j].id;
            float ln = 0.0f, lt = 0.0f;
            for (int q = 0; q < g.point_count && q < 2; ++q)
                if (g.points[q].id == id) { ln = g.points[q].normal_impulse; lt = g.points[q].tangent_impulse; }
            ln = ln > 0.0f ? ln : 0.0f;
            const float mf = vr.K.w * ln;
            lt = lt < -mf ? -mf : (lt > mf ? mf : lt);
            if (j == 0) { vr.imp.x = ln; vr.imp.y = lt; }
            else { vr.imp.z = ln; vr.imp.w = lt; }
        }
    }
    return x.ws_mode == 2;
}

// Predicted start impulses for pending rows pend[p0 .. p0 + 16) (of npend), one warp, one
// tensor-core pass: features normalised into X (16 x kFeat bf16), the network's hidden layers
// in H1 / H2 (16 x kHid bf16 each), the new points' impulses clamped as the solver could reach
// them (normal >= 0, |tangent| <= friction * normal) and the rows marked predicted (0x100)
DG void infer_pending16(const Ctx& x, const int* pend, int p0, int npend, VRow* vrow, __nv_bfloat16* X,
                        __nv_bfloat16* H1, __nv_bfloat16* H2) {
    const int lane = lane_id();
    for (int e = lane; e < 16 * kFeat; e += kWarp) {
        int r = e / kFeat, q = e % kFeat;
        float v = 0.0f;
        if (p0 + r < npend) {
            int item = vrow[pend[p0 + r]].ids.w;
            v = (x.s_feat[(size_t)kFeat * item + q] - x.mlp.fmean[q]) / x.mlp.fstd[q];
        }
        X[e] = __float2bfloat16_rn(v);
    }
    __syncwarp();
    float y[4];
    mlp_infer16(x.mlp, X, H1, H2, y, lane);
    __syncwarp();
    const int g = lane >> 2, t = lane & 3;
    if (t < 2) {
#pragma unroll
        for (int hrow = 0; hrow < 2; ++hrow) {
            const int r = g + 8 * hrow;
            if (p0 + r >= npend) continue;
            const int idx = pend[p0 + r];
            VRow* vr = vrow + idx;
            const int ids = vr->ids.z;
            const int j = t;                              // lane t predicts point t
            if (!(ids & (0x200 << j)) || j >= (ids & 0xff)) continue;
            const int c = 2 * t;
            float ln = y[2 * hrow] * x.mlp.tstd[c] + x.mlp.tmean[c];
            float lt = y[2 * hrow + 1] * x.mlp.tstd[c + 1] + x.mlp.tmean[c + 1];
            ln = ln > 0.0f ? ln : 0.0f;                   // a start the solver itself could reach
            float mf = vr->K.w * ln;
            lt = lt < -mf ? -mf : (lt > mf ? mf : lt);
            if (j == 0) { vr->imp.x = ln; vr->imp.y = lt; }
            else { vr->imp.z = ln; vr->imp.w = lt; }
        }
    }
    if (t == 0) {
        for (int hrow = 0; hrow < 2; ++hrow) {
            const int r = g + 8 * hrow;
            if (p0 + r < npend) atomicOr(&vrow[pend[p0 + r]].ids.z, 0x100);
        }
    }
    __syncwarp();
}

// deepest separation over the points of a contact at the current positions
// (b2PositionSolverManifold, b2contactsolver.d:816-851); 0 when none is below 0
DG float position_min_separation(const PC& pc, SB sb) {
    float2 cA = sb.c(pc.bodyA), cB = sb.c(pc.bodyB);
    Xf xfA, xfB;
    xfA.q = rot(sb.a(pc.bodyA));
    xfB.q = rot(sb.a(pc.bodyB));
    xfA.p = cA - mul(xfA.q, pc.lcA);
    xfB.p = cB - mul(xfB.q, pc.lcB);
    float minSep = 0.0f;
    for (int j = 0; j < pc.pointCount; ++j) {
        float separation;
        if (pc.type == kManifoldCircles) {
            float2 pointA = mul(xfA, pc.localPoint), pointB = mul(xfB, pc.localPoints[0]);
            float2 normal = pointB - pointA;
            normalize(normal);
            separation = (dot(pointB - pointA, normal) - pc.radiusA) - pc.radiusB;
        } else {
            bool faceA = pc.type == kManifoldFaceA;
            Xf xfN = faceA ? xfA : xfB, xfC = faceA ? xfB : xfA;
            float2 normal = mul(xfN.q, pc.localNormal);
            float2 planePoint = mul(xfN, pc.localPoint), clipPoint = mul(xfC, pc.localPoints[j]);
            separation = (dot(clipPoint - planePoint, normal) - pc.radiusA) - pc.radiusB;
        }
        minSep = bmin(minSep, separation);
    }
    return minSep;
}

// Level offsets of a schedule (lvl[0 .. last]) held in registers: lane k of q0 / q1 / q2
// has lvl[32 * (blk + j) + k].  The level being solved and the levels read ahead of it
// are at most one block apart, so each offset is one shuffle away, and the block after
// next is loaded 32 levels before it is needed.
struct LevelQ {
    const int* lvl;
    int last, blk, q0, q1, q2;
    DG int ld(int i) const { return i <= last ? lvl[i] : 0; }
    DG void init(const int* l, int last_) {
        lvl = l; last = last_; blk = 0;
        int lane = lane_id();
        q0 = ld(lane); q1 = ld(32 + lane); q2 = ld(64 + lane);
    }
    DG void step_to(int L) {
        while ((L >> 5) > blk) { ++blk; q0 = q1; q1 = q2; q2 = ld(32 * (blk + 2) + lane_id()); }
    }
    DG int get(int i) const {
        int a = __shfl_sync(0xffffffffu, q0, i & 31), b = __shfl_sync(0xffffffffu, q1, i & 31);
        return (i >> 5) == blk ? a : b;
    }
};

template <class F>
DG void run_levels(const int* lvl, int maxL, F&& f) {
    LevelQ q;
    q.init(lvl, maxL + 1);
    const int lane = lane_id();
    for (int L = 1; L <= maxL; ++L) {
        q.step_to(L);
        int s = q.get(L), e = q.get(L + 1);
        if (s + lane < e) f(s + lane);
        if (e - s > kWarp)
            for (int idx = s + lane + kWarp; idx < e; idx += kWarp) f(idx);
        tsync();
    }
}

DG VRow load_row(const VRow* p) { return load_v(p); }
DG PRow load_row(const PRow* p) { return load_p(p); }

// ---- bulk staging of constraint rows (one-dimensional TMA copies completed on mbarriers)
DG unsigned smem_u32(const void* p) { return (unsigned)__cvta_generic_to_shared(p); }
DG void mbar_init(unsigned long long* bar) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" :: "r"(smem_u32(bar)) : "memory");
}
DG void fence_mbar_init() { asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory"); }
DG void fence_async_shared() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }
DG void fence_async_global() { asm volatile("fence.proxy.async.global;" ::: "memory"); }
// arm `bar` for `bytes` and copy them global -> shared; completes the barrier's phase
DG void bulk_copy(unsigned long long* bar, void* dst, const void* src, unsigned bytes) {
    unsigned b = smem_u32(bar);
    asm volatile("{\n\t.reg .b64 st;\n\tmbarrier.arrive.expect_tx.shared::cta.b64 st, [%0], %1;\n\t}"
                 :: "r"(b), "r"(bytes) : "memory");
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];"
                 :: "r"(smem_u32(dst)), "l"(src), "r"(bytes), "r"(b) : "memory");
}
constexpr int kMbarSpinLimit = 1 << 20;
// Wait for the phase of `bar` with the given parity.  `budget` polls is what the wait may take
// (Ctx.wait_polls, kMbarSpinLimit unless a caller lowers it): past it the wait is reported
// (false) but keeps polling, up to kMbarSpinLimit polls in all, so that the copy has landed
// before its rows are read and no copy is still in flight when the block exits.  Only a copy
// that never completes within kMbarSpinLimit polls leaves stale (in-bounds) rows behind.
DG bool mbar_wait(unsigned long long* bar, unsigned parity, int budget) {
    unsigned b = smem_u32(bar);
    for (int i = 0; i < kMbarSpinLimit; ++i) {
        unsigned done;
        asm volatile("{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
                     "selp.u32 %0, 1, 0, p;\n\t}" : "=r"(done) : "r"(b), "r"(parity) : "memory");
        if (done) return i < budget;
    }
    return false;
}

// Row staging of one warp: a ring of two halves in shared memory, each one block of
// consecutive schedule positions (32 velocity rows or 48 position rows, 4608 bytes), with
// one mbarrier per half.  `par` holds the phase bit each half waits for next.
struct RowRing {
    float* base;                   // 9216 bytes of rows
    unsigned long long* bar;       // two mbarriers
    unsigned par;
    bool ok;                       // no wait went past its budget
    int budget;                    // polls a wait may take (Ctx.wait_polls)
};

// One sweep over levels 1..maxL of a schedule whose rows are stored in schedule order:
// f(row, idx) for every position of a level, levels in order, positions of a level spread
// over the lanes.  Rows arrive by blocks: block m+1 is copied by one bulk copy as soon as
// the sweep reaches block m, so a level reads its rows from shared memory and the copies
// stay off the dependent chain between levels.  A level wider than the warp runs as chunks
// of 32 positions with a warp sync between them (positions of a level are independent, so
// any split keeps the result); a chunk spans at most two consecutive blocks, which are
// both resident.  A row of a later position is never written by an earlier level, and the
// rows' global writes of the previous sweep are ordered before the copies by the proxy
// fence at the start.  f has one call site, which keeps the loop small in the instruction
// cache.
template <class RowT, class F>
DG void sweep_levels(const int* lvl, int maxL, int nItems, const RowT* rows, RowRing& ring, F&& f) {
    if (maxL < 1) return;
    constexpr int B = (int)(4608 / sizeof(RowT));
    static_assert(4608 % sizeof(RowT) == 0 && sizeof(RowT) % 16 == 0, "rows tile a half of the ring");
    static_assert(B >= kWarp, "a chunk spans at most two blocks");
    const int lane = lane_id();
    RowT* slots = reinterpret_cast<RowT*>(ring.base);
    const int nblk = (nItems + B - 1) / B;
    int issued = -1, waited = -1;
    auto wait_next = [&]() {
        ++waited;
        const int h = waited & 1;
        ring.ok &= mbar_wait(&ring.bar[h], (ring.par >> h) & 1u, ring.budget);
        ring.par ^= 1u << h;
    };
    auto issue_upto = [&](int want) {
        want = want < nblk - 1 ? want : nblk - 1;
        while (issued < want) {
            const int m = issued + 1;
            while (waited < m - 2) wait_next();          // the half's previous block has landed
            if (lane == 0) {
                fence_async_shared();
                int cnt = nItems - m * B;
                cnt = cnt < B ? cnt : B;
                bulk_copy(&ring.bar[m & 1], slots + (m & 1) * B, rows + (size_t)m * B, (unsigned)(cnt * sizeof(RowT)));
            }
            issued = m;
        }
    };
    fence_async_global();                                // this lane's row writes before the copies
    tsync();
    issue_upto(1);
    // level ends two levels ahead in registers (plain loads; their latency hides behind a level)
    auto off = [&](int i) { return i <= maxL + 1 ? lvl[i] : nItems; };
    int s = off(1), e = off(2), e2 = off(3);
    // the bookkeeping runs only when a chunk reaches a block that is not yet waited for or
    // passes the point where the next block is issued
    int t_wait = 0, t_issue = 0;
    for (int L = 1; L <= maxL;) {
        const int e3 = off(L + 3);
        const int ce = e - s > kWarp ? s + kWarp : e;    // end of this chunk of the level
        if (ce > t_wait || s >= t_issue) {
            const int mlo = s / B;
            issue_upto(mlo + 1);
            const int mneed = (ce - 1) / B;
            while (waited < mneed) wait_next();
            t_wait = (waited + 1) * B;
            t_issue = issued < nblk - 1 ? issued * B : 0x7fffffff;
        }
        if (s + lane < ce) {
            const int idx = s + lane;
            f(slots[idx % (2 * B)], idx);
        }
        tsync();
        const bool next_level = ce == e;
        s = ce;
        L += next_level;
        e = next_level ? e2 : e;
        e2 = next_level ? e3 : e2;
    }
    while (waited < issued) wait_next();
}


// b2World.Solve (b2world.d:930-1124) for world w: islands, contact solver, sleep,
// SynchronizeFixtures, FindNewContacts.  sbp: the world's solver body rows; stage_f: this
// warp's staging area in shared memory; ring: the warp's row ring in that area, whose
// barriers are initialised once per launch and carry their phases from world to world.
DG void solve_world(const Ctx& x, int w, float* sbp, bool sb_smem, float* stage_f, RowRing& ring) {
    const WorldInfo& wi = x.wi[w];
    WorldDyn& wd = x.wd[w];
    int lane = lane_id();
    if (!(wd.step_complete && x.dt > 0.0f)) return;
    const int b0 = wi.body_start, nb = wi.body_count;
    const int c0 = wi.contact_start, n = wd.contact_count;
    const int j0 = wi.joint_start, nj = wi.joint_count;
    const int bx = wi.bx_start, kx = wi.kx_start;
    const float h = x.dt;
    const bool warm = x.warm_starting != 0;
    const float dtRatio = wd.inv_dt0 * x.dt;                            // b2world.d:392
    stamp(x, w, 0);
    if (x.measure && lane == 0) { wd.q_sumsq = 0.0f; wd.q_max = 0.0f; wd.q_points = 0; wd.q_minsep = 0.0f; }
    SB sb;
    sb.p = sbp;
    // per-island flags and minimum separations of the position iterations: after the
    // world's body rows in shared memory when those are there, else global rows
    int* iflags = sb_smem ? reinterpret_cast<int*>(sbp + 6 * nb) : x.s_isl_flags + b0;
    unsigned* iminsep = sb_smem ? reinterpret_cast<unsigned*>(sbp + 7 * nb) : x.s_isl_minsep + b0;
    ring.ok = true;
    unsigned char* bfl = x.s_bfl + b0;
    // compact per-body / per-contact data; island flags cleared (b2world.d:944-957)
    for (int i = lane; i < nb; i += kWarp) {
        dbox_body_state& B = x.bs[b0 + i];
        B.flags &= ~(uint32_t)kBodyIsland;
        bfl[i] = body_flag_byte(B);
        x.s_cursor[b0 + i] = 0;
        x.s_body_island[b0 + i] = -1;
        sb_load(sb, i, B);
    }
    // scratch of the island search: this warp's staging area when the world fits, else
    // global rows: edge counts / adjacency starts, the DFS stack (later the per-body last
    // level of the schedule), body flag bytes and contact visit marks
    const int nbA = (nb + 4) & ~3;
    const bool gsm = 4 * (nb + 1) + 4 * nb + nbA + ((n + 3) & ~3) <= (int)(kStageFloats * sizeof(float));
    int* adj = gsm ? reinterpret_cast<int*>(stage_f) : x.s_adj_start + bx;
    int* stack = gsm ? adj + nb + 1 : x.s_stack + b0;
    unsigned char* vbf = gsm ? reinterpret_cast<unsigned char*>(stack + nb) : bfl;
    unsigned char* cvis = gsm ? vbf + nbA : x.s_cvis + c0;
    for (int i = lane; i < nb; i += kWarp) {
        adj[i] = 0;
        if (gsm) vbf[i] = bfl[i];
    }
    for (int k = lane; k < n; k += kWarp) {
        x.ct[c0 + k].flags &= ~(uint32_t)kContactIsland;
        contact_compact(x, c0 + k, b0);
        cvis[k] = 0;
    }
    for (int j = lane; j < nj; j += kWarp) x.jt[j0 + j].island_flag = 0;
    tsync();
    // contact edges of the island graph per body (b2world.d:1026-1062 walks them newest first)
    for (int k = lane; k < n; k += kWarp) {
        if (x.s_cq[c0 + k] & 1) {
            int2 cb = x.s_cbody[c0 + k];
            atomicAdd(&adj[cb.x], 1);
            atomicAdd(&adj[cb.y], 1);
        }
    }
    tsync();
    {
        int total = 0;
        for (int base = 0; base < nb; base += kWarp) {
            int i = base + lane;
            int v = i < nb ? adj[i] : 0;
            int incl = v;
            for (int o = 1; o < 32; o <<= 1) {
                int t = __shfl_up_sync(0xffffffffu, incl, o);
                if (lane >= o) incl += t;
            }
            if (i < nb) { adj[i] = total + incl - v; stack[i] = total + incl - v; }
            total += __shfl_sync(0xffffffffu, incl, 31);
        }
        if (lane == 0) adj[nb] = total;
    }
    tsync();
    // adjacency lists, newest contact first: 32 contacts at a time, lane 0 the newest; an
    // edge's place is its body's running count plus the newer edges of that body in the batch
    int2* items = x.s_adj_items + 2 * (size_t)c0;
    for (int top = n - 1; top >= 0; top -= kWarp) {
        int k = top - lane;
        bool edge = k >= 0 && (x.s_cq[c0 + k] & 1);
        int2 cb = edge ? x.s_cbody[c0 + k] : make_int2(-1, -1);
        int rA = 0, rB = 0;
#pragma unroll 8
        for (int j = 0; j < kWarp; ++j) {
            int oa = __shfl_sync(0xffffffffu, cb.x, j), ob = __shfl_sync(0xffffffffu, cb.y, j);
            if (j < lane && oa >= 0) {
                rA += (oa == cb.x) + (ob == cb.x);
                rB += (oa == cb.y) + (ob == cb.y);
            }
        }
        int pA = 0, pB = 0;
        if (edge) { pA = stack[cb.x] + rA; pB = stack[cb.y] + rB; }
        tsync();
        if (edge) {
            items[pA] = make_int2(k, cb.y);
            items[pB] = make_int2(k, cb.x);
            atomicAdd(&stack[cb.x], 1);
            atomicAdd(&stack[cb.y], 1);
        }
        tsync();
    }
    stamp(x, w, 1);
    int nIsl = 0, nbI = 0, ncI = 0, njI = 0, maxLv = 0, maxLp = 0;
    {
        int* statics = x.s_last + b0;
        int* isl_body = x.s_isl_body + b0;
        int* isl_contact = x.s_isl_contact + c0;
        int2* isl_pair = x.s_isl_pair + c0;
        int* body_island = x.s_body_island + b0;
        // depth-first island search (b2world.d:959-1095), seeds in list order (descending index).
        // The whole warp runs it: a popped body's edges are taken 32 at a time, each lane one
        // edge; the contacts not yet in an island are appended in edge order, and the bodies
        // they reach that are not yet marked are pushed in edge order (a body reached twice in
        // the same 32 edges by its first edge only), which is what the reference's one-edge-
        // at-a-time loop does.  Joint edges (rarer) are walked by lane 0.
        const unsigned lt = (1u << lane) - 1u;
        auto dfs_seed = [&](int seed) {
            unsigned char fs = vbf[seed];
            if (fs & kBfVisited) return;
            if ((fs & kBfAwake) == 0 || (fs & kBfActive) == 0) return;
            if (fs & kBfStatic) return;
            if (lane == 0) {
                x.s_isl_bstart[bx + nIsl] = nbI;
                x.s_isl_cstart[bx + nIsl] = ncI;
                x.s_isl_jstart[bx + nIsl] = njI;
                stack[0] = seed;
                vbf[seed] = fs | kBfVisited;
            }
            int top = 1, nStatic = 0;
            tsync();
            while (top > 0) {
                const int b = stack[--top];
                const unsigned char fb = vbf[b];
                tsync();
                if (lane == 0) body_island[b] = nIsl;
                if (fb & kBfStatic) {
                    if (lane == 0) statics[nStatic] = b;
                    ++nStatic;
                    continue;
                }
                if (lane == 0) { isl_body[nbI] = b; vbf[b] = fb | kBfPopped; }
                ++nbI;
                for (int e0 = adj[b], ee = adj[b + 1]; e0 < ee; e0 += kWarp) {
                    const int e = e0 + lane;
                    int2 it = make_int2(0, 0);
                    bool newc = false;
                    unsigned char fo = kBfVisited;
                    if (e < ee) {
                        it = items[e];
                        // in an island already exactly when the other body is non-static and
                        // was popped before (its walk added the contact)
                        fo = vbf[it.y];
                        newc = (fo & (kBfPopped | kBfStatic)) != kBfPopped;
                    }
                    const unsigned cm = __ballot_sync(0xffffffffu, newc);
                    if (newc) {
                        const int pos = ncI + __popc(cm & lt);
                        isl_contact[pos] = c0 + it.x;
                        isl_pair[pos] = make_int2(b, it.y);
                        cvis[it.x] = 1;
                    }
                    ncI += __popc(cm);
                    const bool cand = newc && !(fo & kBfVisited);
                    const unsigned same = __match_any_sync(0xffffffffu, cand ? it.y : -1 - lane);
                    const bool push = cand && (__ffs(same) - 1) == lane;
                    const unsigned pm = __ballot_sync(0xffffffffu, push);
                    if (push) {
                        stack[top + __popc(pm & lt)] = it.y;
                        vbf[it.y] = fo | kBfVisited;
                    }
                    top += __popc(pm);
                    tsync();
                }
                if (nj == 0) continue;
                if (lane == 0) {
                    const BodyStatic& st = x.bst[b0 + b];
                    for (int e = 0; e < st.jadj_count; ++e) {
                        int j = x.jadj_joint[st.jadj_start + e];
                        if (x.jt[j].island_flag) continue;
                        int other = x.jadj_other[st.jadj_start + e] - b0;
                        unsigned char fo = vbf[other];
                        if ((fo & kBfActive) == 0) continue;
                        x.s_isl_joint[j0 + njI++] = j;
                        x.jt[j].island_flag = 1;
                        if (fo & kBfVisited) continue;
                        stack[top++] = other;
                        vbf[other] = fo | kBfVisited;
                    }
                }
                top = __shfl_sync(0xffffffffu, top, 0);
                njI = __shfl_sync(0xffffffffu, njI, 0);
                tsync();
            }
            for (int i = lane; i < nStatic; i += kWarp) vbf[statics[i]] &= ~kBfVisited;
            tsync();
            ++nIsl;
        };
        // 32 seeds at a time: a seed with no island contact and no joint is an island of its
        // own that no other search reaches, so when every seed that starts an island in the
        // chunk is such a body the lanes write those islands at once; otherwise lane 0 walks
        // the chunk seed by seed
        for (int base = nb - 1; base >= 0; base -= kWarp) {
            const int sd = base - lane;
            const unsigned char fs = sd >= 0 ? vbf[sd] : (unsigned char)kBfVisited;
            const bool elig = sd >= 0 && !(fs & kBfVisited) && (fs & kBfAwake) && (fs & kBfActive) && !(fs & kBfStatic);
            const bool lone = elig && adj[sd] == adj[sd + 1] && (nj == 0 || x.bst[b0 + sd].jadj_count == 0);
            const unsigned em = __ballot_sync(0xffffffffu, elig), lm = __ballot_sync(0xffffffffu, lone);
            if (em == lm) {
                if (lone) {
                    const int k = __popc(lm & ((1u << lane) - 1u));
                    x.s_isl_bstart[bx + nIsl + k] = nbI + k;
                    x.s_isl_cstart[bx + nIsl + k] = ncI;
                    x.s_isl_jstart[bx + nIsl + k] = njI;
                    body_island[sd] = nIsl + k;
                    isl_body[nbI + k] = sd;
                    vbf[sd] = fs | kBfVisited;
                }
                nIsl += __popc(lm);
                nbI += __popc(lm);
                tsync();
                continue;
            }
            tsync();
            for (int seed = base; seed > base - kWarp && seed >= 0; --seed) dfs_seed(seed);
            tsync();
        }
        if (lane == 0) {
            x.s_isl_bstart[bx + nIsl] = nbI;
            x.s_isl_cstart[bx + nIsl] = ncI;
            x.s_isl_jstart[bx + nIsl] = njI;
            wd.islands = nIsl;
        }
    }
    nIsl = __shfl_sync(0xffffffffu, nIsl, 0);
    nbI = __shfl_sync(0xffffffffu, nbI, 0);
    ncI = __shfl_sync(0xffffffffu, ncI, 0);
    njI = __shfl_sync(0xffffffffu, njI, 0);
    tsync();
    stamp(x, w, 2);
    if (gsm)
        for (int i = lane; i < nb; i += kWarp) bfl[i] = vbf[i];
    for (int k = lane; k < n; k += kWarp)
        if (cvis[k]) x.ct[c0 + k].flags |= kContactIsland;
    // level schedules; without joints in the islands the two orders coincide and one
    // schedule serves both
    int* last = gsm ? stack : x.s_last + b0;
    maxLv = build_schedule(x, wi, nIsl, false, vbf, last, x.s_sched_v, x.s_lvl_v);
    int* sched_p = x.s_sched_v;
    int* lvl_p = x.s_lvl_v;
    maxLp = maxLv;
    if (njI) {
        sched_p = x.s_sched_p;
        lvl_p = x.s_lvl_p;
        maxLp = build_schedule(x, wi, nIsl, true, vbf, last, sched_p, lvl_p);
    }
    if (x.prof && lane == 0) { x.prof[kProfSlots * (size_t)w + 12] = maxLv; x.prof[kProfSlots * (size_t)w + 13] = n; x.prof[kProfSlots * (size_t)w + 14] = nb; }
    stamp(x, w, 3);
    if (lane == 0) {
        wd.acc_isl_bodies += (unsigned long long)nbI;
        wd.acc_isl_contacts += (unsigned long long)ncI;
        wd.acc_vsolve += (unsigned long long)ncI * (unsigned long long)x.vel_iters;
    }
    tsync();
    // island flags and SetAwake(true) of the search (b2world.d:985-1004), applied after it
    for (int i = lane; i < nb; i += kWarp) {
        dbox_body_state& B = x.bs[b0 + i];
        if ((bfl[i] & kBfVisited) && !(bfl[i] & kBfStatic)) B.flags |= kBodyIsland;
        if (x.s_body_island[b0 + i] >= 0) b_set_awake(B, true);
    }
    // integrate velocities (b2island.d:82-116)
    for (int t = lane; t < nbI; t += kWarp) {
        int i = x.s_isl_body[b0 + t];
        dbox_body_state& B = x.bs[b0 + i];
        B.sweep[2] = B.sweep[4];
        B.sweep[3] = B.sweep[5];
        B.sweep[6] = B.sweep[7];
        if (B.type == kDynamicBody) {
            const BodyStatic& st = x.bst[b0 + i];
            float2 v = sb.v(i);
            float wv = sb.w(i);
            float2 g = st.gravity_scale * x.gravity + B.mass[1] * v2(B.force[0], B.force[1]);
            v += h * g;
            wv += (h * B.mass[3]) * B.force[2];
            v *= fdiv(1.0f, 1.0f + h * st.lin_damping);
            wv *= fdiv(1.0f, 1.0f + h * st.ang_damping);
            sb.set_v(i, v, wv);
        }
    }
    tsync();
    // constraint rows in schedule order: b2ContactSolver ctor + InitializeVelocityConstraints
    // (b2contactsolver.d:244-450); joint positions carry only the joint index
    const int nItems = ncI + njI;
    VRow* vrow = x.vr + kx;
    PRow* prow = x.pr + kx;
    int npend = 0;                                   // learned start: contacts waiting for a prediction
    for (int base = 0; base < nItems; base += kWarp) {
        const int idx = base + lane;
        bool pend = false;
        if (idx < nItems) {
            int item = x.s_sched_v[kx + idx];
            bool pdone = false;
            if (item >= 0) {
                VC vc;
                PC pc;
                constraint_ctor(x, item, b0, warm, dtRatio, vc, pc);
                float sep[2] = {0.0f, 0.0f};
                constraint_init_velocity(vc, pc, sb, sep);
                VRow vr = pack_v(vc, item);
                if (x.ws_mode) pend = row_start_modes(x, item, kx + idx, vc, pc, sep, sb, h, vr);
                vrow[idx] = vr;
                if (njI || x.record_events) x.s_vpos[item] = idx;
                if (!njI) {
                    // one schedule serves both orders: the position row of this place is this contact's
                    prow[idx] = pack_p(pc, x.s_body_island[b0 + ((bfl[vc.bodyA] & kBfStatic) ? vc.bodyB : vc.bodyA)]);
                    pdone = true;
                }
            } else {
                vrow[idx].ids = make_int4(0, 0, 0, item);
                if (x.ws_mode == 1) x.s_slog[kx + idx] = -1;
            }
            if (!pdone) {
                int pitem = sched_p[kx + idx];
                int is = item_island(x, pitem, b0);
                if (pitem >= 0) {
                    VC vc;
                    PC pc;
                    constraint_ctor(x, pitem, b0, warm, dtRatio, vc, pc);
                    prow[idx] = pack_p(pc, is);
                } else {
                    prow[idx].ids = make_int4(0, 0, pitem, is);
                }
            }
        }
        if (x.ws_mode == 2) {
            unsigned bal = __ballot_sync(0xffffffffu, pend);
            if (pend) x.s_pend[c0 + npend + __popc(bal & ((1u << lane) - 1u))] = idx;
            npend += __popc(bal);
        }
    }
    tsync();
    // learned start: predicted impulses for the new points, 16 contacts per tensor-core pass,
    // in this warp's staging area (free until the sweeps)
    for (int p0 = 0; p0 < npend; p0 += 16) {
        __nv_bfloat16* X = reinterpret_cast<__nv_bfloat16*>(stage_f);
        infer_pending16(x, x.s_pend + c0, p0, npend, vrow, X, X + 16 * kFeat, X + 16 * kFeat + 16 * kHid);
    }
    tsync();
    stamp(x, w, 4);
    // warm start contacts, then joints' InitVelocityConstraints (b2island.d:133-146)
    if (njI == 0) {
        // without joints the position-order and velocity-order schedules coincide
        if (warm)
            sweep_levels(x.s_lvl_v + kx, maxLv, nItems, vrow, ring, [&](const VRow& r, int) { warm_start(unpack_v(r), sb); });
    } else {
        run_levels(lvl_p + kx, maxLp, [&](int idx) {
            int item = sched_p[kx + idx];
            if (item >= 0) { if (warm) warm_start(unpack_v(load_v(vrow + x.s_vpos[item])), sb); }
            else joint_init(x, -item - 1, b0, sb, warm, dtRatio);
        });
    }
    stamp(x, w, 5);
    // velocity iterations (b2island.d:153-161)
    auto contact_velocity = [&](const VRow& r, int idx) {
        VC vc = unpack_v(r);
        BodyVel q = load_vel(sb, vc.bodyA, vc.bodyB);
        if (vc.pointCount == 2) solve_velocity_two(vc, q);
        else solve_velocity(vc, q);
        store_vel(sb, vc.bodyA, vc.bodyB, q);
        vrow[idx].imp = make_float4(vc.p[0].normalImpulse, vc.p[0].tangentImpulse, vc.p[1].normalImpulse,
                                    vc.p[1].tangentImpulse);
    };
    for (int it = 0; it < x.vel_iters; ++it) {
        if (njI == 0 && !(it == 0 && x.ws_mode == 2)) {
            // contacts only, no learned first iteration: the row needs no kind test
            sweep_levels(x.s_lvl_v + kx, maxLv, nItems, vrow, ring, contact_velocity);
            continue;
        }
        sweep_levels(x.s_lvl_v + kx, maxLv, nItems, vrow, ring, [&](const VRow& r, int idx) {
            if (r.ids.w >= 0) {
                if (it == 0 && (r.ids.z & 0x100)) {
                    float4 im;
                    solve_velocity_learned(r, sb, &im);
                    vrow[idx].imp = im;
                    return;
                }
                contact_velocity(r, idx);
            } else {
                joint_solve_velocity(x, -r.ids.w - 1, b0, sb);
            }
        });
    }
    stamp(x, w, 6);
    if (x.measure) {
        // one extra velocity sweep that changes nothing: the bodies' velocities are kept
        // aside and put back, impulses are not written, joints are left out
        for (int t = lane; t < nbI; t += kWarp) {
            int i = x.s_isl_body[b0 + t];
            float2 v = sb.v(i);
            x.s_vsave[3 * (size_t)(b0 + i)] = v.x;
            x.s_vsave[3 * (size_t)(b0 + i) + 1] = v.y;
            x.s_vsave[3 * (size_t)(b0 + i) + 2] = sb.w(i);
        }
        tsync();
        float ssq = 0.0f, smax = 0.0f;
        int npts = 0;
        sweep_levels(x.s_lvl_v + kx, maxLv, nItems, vrow, ring, [&](const VRow& r, int) {
            if (r.ids.w < 0) return;
            VC vc = unpack_v(r);
            VC before = vc;
            solve_velocity(vc, sb);
            for (int j = 0; j < vc.pointCount; ++j) {
                float dn = vc.p[j].normalImpulse - before.p[j].normalImpulse;
                float dt = vc.p[j].tangentImpulse - before.p[j].tangentImpulse;
                float d2 = dn * dn + dt * dt;
                ssq += d2;
                smax = bmax(smax, sqrtf(d2));
                ++npts;
            }
        });
        for (int o = 16; o > 0; o >>= 1) {
            ssq += __shfl_xor_sync(0xffffffffu, ssq, o);
            smax = bmax(smax, __shfl_xor_sync(0xffffffffu, smax, o));
            npts += __shfl_xor_sync(0xffffffffu, npts, o);
        }
        if (lane == 0) { wd.q_sumsq = ssq; wd.q_max = smax; wd.q_points = npts; }
        tsync();
        for (int t = lane; t < nbI; t += kWarp) {
            int i = x.s_isl_body[b0 + t];
            const float* sv = x.s_vsave + 3 * (size_t)(b0 + i);
            sb.set_v(i, v2(sv[0], sv[1]), sv[2]);
        }
        tsync();
    }
    for (int idx = lane; idx < nItems; idx += kWarp) {
        VRow r = load_v(vrow + idx);
        if (r.ids.w >= 0) store_impulses(x, r);
        if (x.ws_mode == 1) {
            int slot = x.s_slog[kx + idx];
            if (slot >= 0) {
                float* tg = x.samples + (size_t)kSampleFloats * slot + kFeat;
                tg[0] = r.imp.x; tg[1] = r.imp.y; tg[2] = r.imp.z; tg[3] = r.imp.w;
            }
        }
    }
    // integrate positions (b2island.d:168-200)
    for (int t = lane; t < nbI; t += kWarp) {
        int i = x.s_isl_body[b0 + t];
        float2 c = sb.c(i);
        float a = sb.a(i);
        float2 v = sb.v(i);
        float wv = sb.w(i);
        float2 translation = h * v;
        if (dot(translation, translation) > kMaxTranslationSquared) {
            float ratio = fdiv(kMaxTranslation, length(translation));
            v *= ratio;
        }
        float rotation = h * wv;
        if (rotation * rotation > kMaxRotationSquared) {
            float ratio = fdiv(kMaxRotation, babs(rotation));
            wv *= ratio;
        }
        c += h * v;
        a += h * wv;
        sb.set_c(i, c, a);
        sb.set_v(i, v, wv);
    }
    for (int is = lane; is < nIsl; is += kWarp) iflags[is] = 0;
    tsync();
    stamp(x, w, 7);
    // position iterations with per-island early exit (b2island.d:206-224)
    for (int it = 0; it < x.pos_iters; ++it) {
        for (int is = lane; is < nIsl; is += kWarp) {
            iminsep[is] = fkey(0.0f);
            iflags[is] &= ~4;
        }
        tsync();
        sweep_levels(lvl_p + kx, maxLp, nItems, prow, ring, [&](const PRow& r, int) {
            int is = r.ids.w;
            if (iflags[is] & 1) return;
            if (r.ids.z >= 0) {
                float ms = solve_position_row(unpack_p(r), sb);
                atomicMin(&iminsep[is], fkey(ms));
            } else if (!joint_solve_position(x, -r.ids.z - 1, b0, sb)) {
                atomicOr(&iflags[is], 4);
            }
        });
        int psolved = 0;
        for (int is = lane; is < nIsl; is += kWarp)
            if (!(iflags[is] & 1))
                psolved += x.s_isl_cstart[bx + is + 1] - x.s_isl_cstart[bx + is];
        for (int o = 16; o > 0; o >>= 1) psolved += __shfl_xor_sync(0xffffffffu, psolved, o);
        if (lane == 0) wd.acc_psolve += (unsigned long long)psolved;
        bool remaining = false;
        for (int is = lane; is < nIsl; is += kWarp) {
            int f = iflags[is];
            if (f & 1) continue;
            bool contactsOkay = funkey(iminsep[is]) >= -3.0f * kLinearSlop;
            bool jointsOkay = (f & 4) == 0;
            if (contactsOkay && jointsOkay) iflags[is] = f | 1 | 2;
            else remaining = true;
        }
        if (!__any_sync(0xffffffffu, remaining)) break;
        tsync();
    }
    tsync();
    if (!__all_sync(0xffffffffu, ring.ok) && lane == 0) set_error(x, w, DBOX_ERR_TIMEOUT);
    if (x.measure) {
        float ms = 0.0f;
        for (int idx = lane; idx < nItems; idx += kWarp) {
            PRow r = load_p(prow + idx);
            if (r.ids.z >= 0) ms = bmin(ms, position_min_separation(unpack_p(r), sb));
        }
        for (int o = 16; o > 0; o >>= 1) ms = bmin(ms, __shfl_xor_sync(0xffffffffu, ms, o));
        if (lane == 0) wd.q_minsep = ms;
    }
    if (x.record_events) {
        // b2Island.Report (b2island.d:419-438): PostSolve per island contact in island order
        const int e0 = wd.ev_count;
        for (int t = lane; t < ncI; t += kWarp) {
            int item = x.s_isl_contact[c0 + t];
            VRow r = load_v(vrow + x.s_vpos[item]);
            float ni[2] = {r.imp.x, r.imp.z}, ti[2] = {r.imp.y, r.imp.w};
            put_event(x, wi, w, e0 + t, DBOX_EVENT_POSTSOLVE, x.ct[item], r.ids.z & 0xff, ni, ti);
        }
        tsync();
        if (lane == 0) wd.ev_count = e0 + ncI;
        tsync();
    }
    stamp(x, w, 8);
    // copy back + SynchronizeTransform (b2island.d:227-235)
    bool nonfinite = false;
    for (int t = lane; t < nbI; t += kWarp) {
        int i = x.s_isl_body[b0 + t];
        dbox_body_state& B = x.bs[b0 + i];
        float2 c = sb.c(i), v = sb.v(i);
        B.sweep[4] = c.x; B.sweep[5] = c.y; B.sweep[7] = sb.a(i);
        B.vel[0] = v.x; B.vel[1] = v.y; B.vel[2] = sb.w(i);
        b_sync_transform(B);
        nonfinite |= !(isfinite(c.x) && isfinite(c.y) && isfinite(B.sweep[7]) && isfinite(v.x) && isfinite(v.y) &&
                       isfinite(B.vel[2]));
    }
    // the reference has no such check (b2Body asserts IsValid on its setters only); a world
    // whose bodies left the finite range is reported as DBOX_ERR_NAN after the step
    if (__any_sync(0xffffffffu, nonfinite) && lane == 0) set_error(x, w, DBOX_ERR_NAN);
    tsync();
    // sleep (b2island.d:241-279)
    if (x.allow_sleep) {
        const float linTolSqr = kLinearSleepTolerance * kLinearSleepTolerance;
        const float angTolSqr = kAngularSleepTolerance * kAngularSleepTolerance;
        for (int is = lane; is < nIsl; is += kWarp) x.s_isl_sleep[b0 + is] = fkey(kMaxFloat);
        tsync();
        for (int t = lane; t < nbI; t += kWarp) {
            int i = x.s_isl_body[b0 + t];
            dbox_body_state& B = x.bs[b0 + i];
            int is = x.s_body_island[b0 + i];
            if ((B.flags & kBodyAutoSleep) == 0 || B.vel[2] * B.vel[2] > angTolSqr ||
                dot(b_v(B), b_v(B)) > linTolSqr) {
                B.sleep_time = 0.0f;
                atomicMin(&x.s_isl_sleep[b0 + is], fkey(0.0f));
            } else {
                B.sleep_time += h;
                atomicMin(&x.s_isl_sleep[b0 + is], fkey(B.sleep_time));
            }
        }
        tsync();
        for (int is = lane; is < nIsl; is += kWarp) {
            int f = iflags[is];
            if (funkey(x.s_isl_sleep[b0 + is]) >= kTimeToSleep && (f & 2)) iflags[is] = f | 8;
        }
        tsync();
        for (int t = lane; t < nbI; t += kWarp) {
            int i = x.s_isl_body[b0 + t];
            if (iflags[x.s_body_island[b0 + i]] & 8) b_set_awake(x.bs[b0 + i], false);
        }
        // a static body ends in the state its last island left it in
        for (int i = lane; i < nb; i += kWarp) {
            if ((bfl[i] & kBfStatic) && x.s_body_island[b0 + i] >= 0 &&
                (iflags[x.s_body_island[b0 + i]] & 8))
                b_set_awake(x.bs[b0 + i], false);
        }
    }
    tsync();
    stamp(x, w, 9);
    // SynchronizeFixtures for bodies that were in an island (b2world.d:1099-1116); a large
    // world's block does it in k_pairs_block
    if (!wi.pair_block)
        for (int i = lane; i < nb; i += kWarp) {
            int b = b0 + i;
            if ((x.bs[b].flags & kBodyIsland) == 0) continue;
            if (x.bs[b].type == kStaticBody) continue;
            sync_fixtures(x, b);
        }
    tsync();
    stamp(x, w, 10);
    if (!wi.pair_block) {                                               // else k_pairs_block + k_finish_big_block
        hash_rebuild(x, w);
        find_new_contacts(x, w);
    }
    stamp(x, w, 11);
}

// ------------------------------------------------------------ TOI
// contact needs a fresh TOI (b2world.d:1159-1210); bodies from the compact arrays
DG bool toi_needs_bodies(const Ctx& x, int ci, int b0);
DG bool toi_needs(const Ctx& x, int ci, int b0) {
    const dbox_contact_state& c = x.ct[ci];
    if ((c.flags & kContactEnabled) == 0) return false;
    if (c.toi_count > kMaxSubSteps) return false;
    if (c.flags & kContactToi) return false;
    return toi_needs_bodies(x, ci, b0);
}
// the part of toi_needs past the contact's own flags and sub-step count
DG bool toi_needs_bodies(const Ctx& x, int ci, int b0) {
    if (x.s_cq[ci] & 2) return false;
    int2 cb = x.s_cbody[ci];
    const dbox_body_state& bA = x.bs[b0 + cb.x];
    const dbox_body_state& bB = x.bs[b0 + cb.y];
    bool activeA = (bA.flags & kBodyAwake) && bA.type != kStaticBody;
    bool activeB = (bB.flags & kBodyAwake) && bB.type != kStaticBody;
    if (!activeA && !activeB) return false;
    bool collideA = (bA.flags & kBodyBullet) || bA.type != kDynamicBody;
    bool collideB = (bB.flags & kBodyBullet) || bB.type != kDynamicBody;
    if (!collideA && !collideB) return false;
    return true;
}

// contact that can ever need a TOI this step: no sensor, and a static, kinematic or bullet
// body on one side (b2world.d:1172-1188; body types and bullet flags do not change inside a step)
DG bool toi_candidate(const Ctx& x, int ci, int b0) {
    if (x.s_cq[ci] & 2) return false;
    int2 cb = x.s_cbody[ci];
    const dbox_body_state& bA = x.bs[b0 + cb.x];
    const dbox_body_state& bB = x.bs[b0 + cb.y];
    bool collideA = (bA.flags & kBodyBullet) || bA.type != kDynamicBody;
    bool collideB = (bB.flags & kBodyBullet) || bB.type != kDynamicBody;
    return collideA || collideB;
}

// b2Contact.Update inside the TOI loop: wakes are applied immediately (out of line: TOI events
// are rare, and the narrowphase inlined here would double the kernel's collision code)
__device__ __noinline__ void toi_update(const Ctx& x, dbox_contact_state& c, unsigned* evt = nullptr) {
    if (contact_update(x, c, evt, true)) {
        b_set_awake(x.bs[x.fx[c.fixture_a].body], true);
        b_set_awake(x.bs[x.fx[c.fixture_b].body], true);
    }
}

// b2Island.SolveTOI (b2island.d:282-416) on the sub-island in s_isl_body (world-local)
// and s_isl_contact; one lane.  sb holds the island bodies' state for the solve.
__device__ __noinline__ void solve_toi_island(const Ctx& x, int w, const WorldInfo& wi, SB sb, int nbI, int ncI, int toiA, int toiB,
                         float subDt) {
    // one warp: the per-body and per-contact set-up, integration and report over its lanes, the
    // position and velocity iterations (Gauss-Seidel over the island's contacts) on lane 0
    const int lane = lane_id();
    const int b0 = wi.body_start, c0 = wi.contact_start;
    VRow* tv = x.tvr + (size_t)kMaxTOIContacts * w;
    PRow* tp = x.tpr + (size_t)kMaxTOIContacts * w;
    for (int i = lane; i < nbI; i += kWarp) {
        int b = x.s_isl_body[b0 + i];
        sb_load(sb, b, x.bs[b0 + b]);
    }
    for (int t = lane; t < ncI; t += kWarp) {
        VC vc;
        PC pc;
        constraint_ctor(x, x.s_isl_contact[c0 + t], b0, false, 1.0f, vc, pc);
        tp[t] = pack_p(pc, 0);
    }
    __syncwarp();
    if (lane == 0) {
        for (int it = 0; it < 20; ++it) {
            float minSep = 0.0f;
            for (int t = 0; t < ncI; ++t)
                minSep = bmin(minSep, solve_position(unpack_p(load_p(tp + t)), sb, true, toiA, toiB));
            if (minSep >= -1.5f * kLinearSlop) break;
        }
        dbox_body_state& A = x.bs[b0 + toiA];
        dbox_body_state& B = x.bs[b0 + toiB];
        float2 cA = sb.c(toiA), cB = sb.c(toiB);
        A.sweep[2] = cA.x; A.sweep[3] = cA.y; A.sweep[6] = sb.a(toiA);
        B.sweep[2] = cB.x; B.sweep[3] = cB.y; B.sweep[6] = sb.a(toiB);
    }
    __syncwarp();
    for (int t = lane; t < ncI; t += kWarp) {
        int ci = x.s_isl_contact[c0 + t];
        VC vc;
        PC pc;
        constraint_ctor(x, ci, b0, false, 1.0f, vc, pc);
        constraint_init_velocity(vc, pc, sb);
        tv[t] = pack_v(vc, ci);
    }
    __syncwarp();
    if (lane == 0)
        for (int it = 0; it < x.vel_iters; ++it)
            for (int t = 0; t < ncI; ++t) {
                VC vc = unpack_v(load_v(tv + t));
                solve_velocity(vc, sb);
                tv[t].imp = make_float4(vc.p[0].normalImpulse, vc.p[0].tangentImpulse, vc.p[1].normalImpulse,
                                        vc.p[1].tangentImpulse);
            }
    __syncwarp();
    float h = subDt;
    for (int i = lane; i < nbI; i += kWarp) {
        int b = x.s_isl_body[b0 + i];
        dbox_body_state& Bd = x.bs[b0 + b];
        float2 c = sb.c(b);
        float a = sb.a(b);
        float2 v = sb.v(b);
        float wv = sb.w(b);
        float2 translation = h * v;
        if (dot(translation, translation) > kMaxTranslationSquared) {
            float ratio = fdiv(kMaxTranslation, length(translation));
            v *= ratio;
        }
        float rotation = h * wv;
        if (rotation * rotation > kMaxRotationSquared) {
            float ratio = fdiv(kMaxRotation, babs(rotation));
            wv *= ratio;
        }
        c += h * v;
        a += h * wv;
        Bd.sweep[4] = c.x; Bd.sweep[5] = c.y; Bd.sweep[7] = a;
        Bd.vel[0] = v.x; Bd.vel[1] = v.y; Bd.vel[2] = wv;
        b_sync_transform(Bd);
    }
    if (x.record_events) {
        // b2Island.Report at the end of b2Island.SolveTOI (b2island.d:411-416)
        WorldDyn& wd = x.wd[w];
        const int e0 = wd.ev_count;
        for (int q = lane; q < ncI; q += kWarp) {
            VRow r = load_v(tv + q);
            float ni[2] = {r.imp.x, r.imp.z}, ti[2] = {r.imp.y, r.imp.w};
            put_event(x, wi, w, e0 + q, DBOX_EVENT_POSTSOLVE, x.ct[x.s_isl_contact[c0 + q]], r.ids.z & 0xff, ni, ti);
        }
        __syncwarp();
        if (lane == 0) wd.ev_count = e0 + ncI;
    }
    __syncwarp();
}

// b2World.SolveTOI (b2world.d:1127-1452) for world w, then the end of b2World.Step
// `prepared`: a large world whose cluster already ran the passes at the start of SolveTOI
// (toi_begin_cluster): the compaction and flag clears, the candidate list (its length in
// WorldDyn.toi_ncand) and the per-body candidate lists
template <class Team>
DG void toi_world_t(const Ctx& x, int w, float* sbp, const Team& tm, bool prepared = false) {
    const WorldInfo& wi = x.wi[w];
    WorldDyn& wd = x.wd[w];
    const int rk = tm.rank(), ts = tm.size();
    const int b0 = wi.body_start, nb = wi.body_count, c0 = wi.contact_start;
    // optional profile: slot 16 total cycles, 17 events, 18.. cycles per part of the event loop
    long long tlast = clock64(), t_start = tlast;
    long long tacc[7] = {0, 0, 0, 0, 0, 0, 0};
    auto mark = [&](int part) {
        if (x.prof) { long long t = clock64(); tacc[part] += t - tlast; tlast = t; }
    };
    if (x.continuous && x.dt > 0.0f) {
        bool advanced = wd.step_complete == 0;
        SB sb;
        sb.p = sbp;
        if (!prepared) {
            int n = wd.contact_count;
            for (int k = rk; k < n; k += ts) contact_compact(x, c0 + k, b0);
        }
        if (wd.step_complete && !prepared) {                             // b2world.d:1131-1146
            for (int i = rk; i < nb; i += ts) {
                x.bs[b0 + i].flags &= ~(uint32_t)kBodyIsland;
                x.bs[b0 + i].sweep[8] = 0.0f;
            }
            int n = wd.contact_count;
            for (int k = rk; k < n; k += ts) {
                dbox_contact_state& c = x.ct[c0 + k];
                c.flags &= ~(uint32_t)(kContactToi | kContactIsland);
                c.toi_count = 0;
                c.toi = 1.0f;
            }
        }
        if (!prepared)
            for (int i = rk; i < nb; i += ts) x.s_bfl[b0 + i] = 0;
        tm.sync();
        // TOI candidates in list order (ascending slot): only these can get a TOI, join a TOI
        // island as a neighbour or carry the TOI / island flags that an event clears
        int* cand = x.s_tcand + c0;
        auto is_cand = [&](int k) { return toi_candidate(x, c0 + k, b0); };
        int ncand = prepared ? wd.toi_ncand : tm.collect(0, wd.contact_count, cand, 0, is_cand);
        // block teams: the candidates of each non-static body (positions in cand, descending),
        // so that an event's joins and invalidations visit only its bodies' candidates; those
        // collected after this point (from the events' new pairs) are scanned apart
        const int ncand0 = ncand;
        int* lstart = x.s_adj_start + wi.bx_start;                       // nb + 1
        int* lent = reinterpret_cast<int*>(x.s_adj_items + 2 * (size_t)c0);
        if constexpr (Team::kLists) if (!prepared) {
            int* lcur = x.s_cursor + b0;
            auto dyn = [&](int b) { return x.bs[b0 + b].type != kStaticBody; };
            for (int i = rk; i < nb; i += ts) lstart[i] = 0;
            tm.sync();
            for (int t = rk; t < ncand; t += ts) {
                const int2 cb = x.s_cbody[c0 + cand[t]];
                if (dyn(cb.x)) atomicAdd(&lstart[cb.x], 1);
                if (dyn(cb.y)) atomicAdd(&lstart[cb.y], 1);
            }
            tm.sync();
            const int tot = block_exclusive_scan(lstart, nb, tm.rl);
            if (tm.lead()) lstart[nb] = tot;
            for (int i = rk; i < nb; i += ts) lcur[i] = lstart[i];
            tm.sync();
            for (int t = rk; t < ncand; t += ts) {
                const int2 cb = x.s_cbody[c0 + cand[t]];
                if (dyn(cb.x)) lent[atomicAdd(&lcur[cb.x], 1)] = t;
                if (dyn(cb.y)) lent[atomicAdd(&lcur[cb.y], 1)] = t;
            }
            tm.sync();
            for (int i = rk; i < nb; i += ts) {                          // each list by descending position
                const int e0 = lstart[i], d = lstart[i + 1] - e0;
                int gap = 1;
                while (3 * gap + 1 < d) gap = 3 * gap + 1;
                for (; gap > 0; gap /= 3)
                    for (int a = e0 + gap; a < e0 + d; ++a) {
                        const int v = lent[a];
                        int q = a - gap;
                        while (q >= e0 && lent[q] < v) { lent[q + gap] = lent[q]; q -= gap; }
                        lent[q + gap] = v;
                    }
            }
            tm.sync();
        }
        // Block teams revisit, after an event, only the candidates whose TOI inputs the event
        // can have changed: those of every body it touched (the event's two bodies, each
        // neighbour a join visited, accepted or not, and both bodies of each new contact, whose
        // AddPair may wake them) and every candidate added since SolveTOI began.  Nothing else
        // changes a candidate's flags, sub-step count or TOI, or the awake state of its bodies.
        // The minimum TOI is kept per 32 consecutive candidates (smallest TOI, then the newest
        // contact slot, which is first in list order) and the chunks holding a revisited
        // candidate are recomputed.  The first event, and any whose revisit list would overflow,
        // take the full passes.
        int* dset = reinterpret_cast<int*>(x.s_isl_pair + c0);          // revisit list (positions)
        const int dcap = 2 * wi.contact_cap;
        int* nlist = x.s_cstate + c0;                                    // the revisited that need a TOI
        unsigned* wmin_a = reinterpret_cast<unsigned*>(x.s_level + wi.kx_start);   // per chunk: TOI bits
        int* wmin_k = x.s_tmp + wi.kx_start;                             // and contact slot (-1: none)
        int* wdirty = x.s_lcur + wi.kx_start;
        int* tbody = x.s_stack + b0;                                     // bodies an event touched
        bool full = true;
        int nd = 0;
        // a large world's event pair searches use the grid of its end-of-solve pair search and
        // the proxies moved since (toi_pairs_big); without destruction a proxy's rank is its
        // fixture index
        const bool big_toi = wi.pair_block && wd.g_valid && !wi.proxy_order;
        const int f0 = wi.fix_start;
        int* toimv = reinterpret_cast<int*>(x.s_sapk[0] + f0);           // moved during this SolveTOI
        int* pnow = x.s_pcount + f0;                                     // moved by this event
        int* pall = x.s_moved + f0;                                      // moved during this SolveTOI
        int nall = 0;
        if (big_toi && !prepared)
            for (int i = rk; i < wi.fix_count; i += ts) toimv[i] = 0;
        tm.sync();
        int events = 0;
        const int max_events = 9 * wi.contact_cap + 16;   // each contact takes at most 9 events
        for (int iter = 0;; ++iter) {
            if (iter >= max_events) {
                if (tm.lead()) set_error(x, w, DBOX_ERR_TIMEOUT);
                break;
            }
            int n = wd.contact_count;
            auto advance_one = [&](int t) {
                const int kk = cand[t];
                const int2 cb = x.s_cbody[c0 + kk];
                dbox_body_state& bA = x.bs[b0 + cb.x];
                dbox_body_state& bB = x.bs[b0 + cb.y];
                float alpha0 = bA.sweep[8];
                if (bA.sweep[8] < bB.sweep[8]) {
                    alpha0 = bB.sweep[8];
                    Sweep s = b_sweep(bA); sweep_advance(s, alpha0); b_set_sweep(bA, s);
                } else if (bB.sweep[8] < bA.sweep[8]) {
                    alpha0 = bA.sweep[8];
                    Sweep s = b_sweep(bB); sweep_advance(s, alpha0); b_set_sweep(bB, s);
                }
                SweepSnap& sn = x.snap[c0 + kk];
                sn.a = b_sweep(bA);
                sn.b = b_sweep(bB);
                sn.alpha0 = alpha0;
            };
            auto compute_toi = [&](int k) {                              // the TOI of a contact that needs one
                dbox_contact_state& c = x.ct[c0 + k];
                const DFixture& fa = x.fx[c.fixture_a];
                const DFixture& fb = x.fx[c.fixture_b];
                Sweep sA, sB;
                float alpha0;
                if (advanced) { sA = x.snap[c0 + k].a; sB = x.snap[c0 + k].b; alpha0 = x.snap[c0 + k].alpha0; }
                else { sA = b_sweep(x.bs[fa.body]); sB = b_sweep(x.bs[fb.body]); alpha0 = sA.alpha0; }
                float beta;
                int state = time_of_impact(make_proxy(fa), make_proxy(fb), sA, sB, 1.0f, &beta);
                float alpha = state == kToiTouching ? bmin(alpha0 + (1.0f - alpha0) * beta, 1.0f) : 1.0f;
                c.toi = alpha;
                c.flags |= kContactToi;
                return alpha;
            };
            float bestA = 1.0f;
            int bestLp = 0x7fffffff;
            bool incremental = false;
            if constexpr (Team::kLists) incremental = !full && advanced;
            if constexpr (Team::kLists) {
              if (incremental) {
                // the revisited candidates that need a TOI, in list order (descending position,
                // repeats dropped) on the lead: sweeps advanced, then their TOIs over the block
                if (tm.lead()) tm.aux[0] = 0;
                tm.sync();
                for (int i = rk; i < nd; i += ts) {
                    const int t = dset[i];
                    if (toi_needs(x, c0 + cand[t], b0)) nlist[atomicAdd(&tm.aux[0], 1)] = t;
                }
                tm.sync();
                int nn = tm.aux[0];
                if (tm.lead()) {
                    for (int a = 1; a < nn; ++a) {                       // descending, few entries
                        const int v = nlist[a];
                        int q = a - 1;
                        while (q >= 0 && nlist[q] < v) { nlist[q + 1] = nlist[q]; --q; }
                        nlist[q + 1] = v;
                    }
                    int m = 0;
                    for (int a = 0; a < nn; ++a)
                        if (m == 0 || nlist[m - 1] != nlist[a]) nlist[m++] = nlist[a];
                    for (int a = 0; a < m; ++a) advance_one(nlist[a]);
                    tm.aux[1] = m;
                }
                tm.sync();
                nn = tm.aux[1];
                mark(0);
                for (int i = rk; i < nn; i += ts) compute_toi(cand[nlist[i]]);
                for (int i = rk; i < nd; i += ts) wdirty[dset[i] >> 5] = 1;
                tm.sync();
                // recompute the chunks that hold a revisited candidate, a warp a chunk: the warps
                // walk the revisit list and the first to claim a chunk's mark recomputes it (the
                // marked chunks are found from the list, not by a walk over every chunk)
                const int nch = (ncand + 31) >> 5, warp = rk >> 5, lane = rk & 31, nw = ts >> 5;
                for (int i = warp; i < nd; i += nw) {
                    const int q = dset[i] >> 5;
                    int claim = 0;
                    if (lane == 0) claim = atomicExch(&wdirty[q], 0);
                    if (!__shfl_sync(0xffffffffu, claim, 0)) continue;
                    const int t = 32 * q + lane;
                    float a = 1.0f;
                    int kb = -1;
                    if (t < ncand) {
                        const int k = cand[t];
                        const dbox_contact_state& c = x.ct[c0 + k];
                        if ((c.flags & kContactEnabled) && c.toi_count <= kMaxSubSteps && (c.flags & kContactToi) &&
                            c.toi < 1.0f) { a = c.toi; kb = k; }
                    }
                    for (int o = 16; o > 0; o >>= 1) {
                        const float oa = __shfl_xor_sync(0xffffffffu, a, o);
                        const int ok = __shfl_xor_sync(0xffffffffu, kb, o);
                        if (oa < a || (oa == a && ok > kb)) { a = oa; kb = ok; }
                    }
                    if (lane == 0) { wmin_a[q] = __float_as_uint(a); wmin_k[q] = kb; }
                }
                tm.sync();
                // the minimum over the chunks (a slot's list position is n - 1 - slot)
                for (int q = rk; q < nch; q += ts) {
                    const int kb = wmin_k[q];
                    if (kb < 0) continue;
                    const float a = __uint_as_float(wmin_a[q]);
                    const int lp = n - 1 - kb;
                    if (a < bestA || (a == bestA && lp < bestLp)) { bestA = a; bestLp = lp; }
                }
                mark(1);
              }
            }
            // sweeps are put onto a common time in list order (b2world.d:1212-1226)
            if (advanced && !incremental) {
                tm.scan_desc(ncand, [&](int t) { return toi_needs(x, c0 + cand[t], b0); }, [&](int t) {
                    const int kk = cand[t];
                    const int2 cb = x.s_cbody[c0 + kk];
                    dbox_body_state& bA = x.bs[b0 + cb.x];
                    dbox_body_state& bB = x.bs[b0 + cb.y];
                    float alpha0 = bA.sweep[8];
                    if (bA.sweep[8] < bB.sweep[8]) {
                        alpha0 = bB.sweep[8];
                        Sweep s = b_sweep(bA); sweep_advance(s, alpha0); b_set_sweep(bA, s);
                    } else if (bB.sweep[8] < bA.sweep[8]) {
                        alpha0 = bA.sweep[8];
                        Sweep s = b_sweep(bB); sweep_advance(s, alpha0); b_set_sweep(bB, s);
                    }
                    SweepSnap& sn = x.snap[c0 + kk];
                    sn.a = b_sweep(bA);
                    sn.b = b_sweep(bB);
                    sn.alpha0 = alpha0;
                    return true;
                });
            }
            if (!incremental) mark(0);
            // the TOI of every contact that needs one (b2world.d:1159-1236), and in the same
            // pass the minimum TOI, first in list order on ties (each contact's TOI is
            // written only by its own iteration)
            // (four candidates of a rank at a time: their slots, then their flags, counts and
            // TOIs are loaded together, and the bodies are read only when the flags leave a
            // fresh TOI possible; block teams also keep each 32-candidate chunk's minimum)
            for (int t0 = rk; (t0 & ~31) < (incremental ? 0 : ncand); t0 += 4 * ts) {
                int kk[4];
                uint32_t fl[4];
                int tc[4];
                float tv[4];
#pragma unroll
                for (int j = 0; j < 4; ++j) kk[j] = t0 + j * ts < ncand ? cand[t0 + j * ts] : -1;
#pragma unroll
                for (int j = 0; j < 4; ++j) {
                    fl[j] = 0u;
                    tc[j] = 0;
                    tv[j] = 1.0f;
                    if (kk[j] >= 0) {
                        const dbox_contact_state& c = x.ct[c0 + kk[j]];
                        fl[j] = c.flags;
                        tc[j] = c.toi_count;
                        tv[j] = c.toi;
                    }
                }
#pragma unroll 1
                for (int j = 0; j < 4; ++j) {
                    const int k = kk[j];
                    bool in = false;
                    if (k >= 0 && (fl[j] & kContactEnabled) && tc[j] <= kMaxSubSteps) {
                        in = true;
                        if ((fl[j] & kContactToi) == 0) {
                            if (toi_needs_bodies(x, c0 + k, b0)) tv[j] = compute_toi(k);
                            else in = false;
                        }
                    }
                    const float toi = tv[j];
                    int lp = n - 1 - k;
                    if (in && (toi < bestA || (toi == bestA && lp < bestLp && toi < 1.0f))) { bestA = toi; bestLp = lp; }
                    if constexpr (Team::kLists) {
                        // this chunk's minimum (all 32 lanes of the warp hold the chunk's candidates)
                        float a = in && toi < 1.0f ? toi : 1.0f;
                        int kb = in && toi < 1.0f ? k : -1;
                        for (int o = 16; o > 0; o >>= 1) {
                            const float oa = __shfl_xor_sync(0xffffffffu, a, o);
                            const int ok = __shfl_xor_sync(0xffffffffu, kb, o);
                            if (oa < a || (oa == a && ok > kb)) { a = oa; kb = ok; }
                        }
                        const int t = t0 + j * ts;
                        if ((rk & 31) == 0 && t < ncand) { wmin_a[t >> 5] = __float_as_uint(a); wmin_k[t >> 5] = kb; wdirty[t >> 5] = 0; }
                    }
                }
            }
            if (!incremental) mark(1);
            tm.argmin(bestA, bestLp);
            mark(2);
            if (bestLp == 0x7fffffff || 1.0f - 10.0f * kEpsilon < bestA) {
                if (tm.lead()) wd.step_complete = 1;
                break;
            }
            const float minAlpha = bestA;
            const int mk = n - 1 - bestLp;
            const int2 mcb = x.s_cbody[c0 + mk];
            int solved = 0, nbI = 0, ncI = 0;
            int ntb = 0;                                                 // bodies this event touched (lead)
            if (tm.lead()) {
                ++events;
                if constexpr (Team::kLists) { tbody[ntb++] = mcb.x; tbody[ntb++] = mcb.y; }
                dbox_contact_state& mc = x.ct[c0 + mk];
                dbox_body_state& bA = x.bs[b0 + mcb.x];
                dbox_body_state& bB = x.bs[b0 + mcb.y];
                Sweep backup1 = b_sweep(bA), backup2 = b_sweep(bB);
                b_advance(bA, minAlpha);
                b_advance(bB, minAlpha);
                unsigned evt = 0;
                toi_update(x, mc, &evt);
                if (x.record_events) put_update_events(x, wi, w, wd, evt, mc);
                mc.flags &= ~(uint32_t)kContactToi;
                ++mc.toi_count;
                if ((mc.flags & kContactEnabled) == 0 || (mc.flags & kContactTouching) == 0) {
                    mc.flags &= ~(uint32_t)kContactEnabled;
                    b_set_sweep(bA, backup1);
                    b_set_sweep(bB, backup2);
                    b_sync_transform(bA);
                    b_sync_transform(bB);
                } else {
                    solved = 1;
                    b_set_awake(bA, true);
                    b_set_awake(bB, true);
                    x.s_isl_body[b0 + nbI++] = mcb.x;
                    x.s_isl_body[b0 + nbI++] = mcb.y;
                    x.s_isl_contact[c0 + ncI++] = c0 + mk;
                    bA.flags |= kBodyIsland;
                    bB.flags |= kBodyIsland;
                    mc.flags |= kContactIsland;
                }
            }
            solved = tm.bcast(solved);
            mark(3);
            if (solved) {
                // contacts of each dynamic event body, in its edge-list order (b2world.d:1306-1411)
                for (int q = 0; q < 2; ++q) {
                    const int body = q == 0 ? mcb.x : mcb.y;
                    if (x.bs[b0 + body].type != kDynamicBody) continue;
                    // every contact that can join (b2world.d:1330-1346) is a candidate
                    auto touches = [&](int t) {
                        const int2 cb = x.s_cbody[c0 + cand[t]];
                        return cb.x == body || cb.y == body;
                    };
                    auto join = [&](int t) {
                        const int kk = cand[t];
                        if (nbI == 2 * kMaxTOIContacts || ncI == kMaxTOIContacts) return false;
                        dbox_body_state& Bd = x.bs[b0 + body];
                        dbox_contact_state& c = x.ct[c0 + kk];
                        if (c.flags & kContactIsland) return true;
                        const int2 cb = x.s_cbody[c0 + kk];
                        const int other = cb.x == body ? cb.y : cb.x;
                        dbox_body_state& O = x.bs[b0 + other];
                        if (O.type == kDynamicBody && (Bd.flags & kBodyBullet) == 0 && (O.flags & kBodyBullet) == 0) return true;
                        if (x.s_cq[c0 + kk] & 2) return true;
                        if constexpr (Team::kLists) { if (ntb < nb) tbody[ntb] = other; ++ntb; }
                        Sweep backup = b_sweep(O);
                        if ((O.flags & kBodyIsland) == 0) b_advance(O, minAlpha);
                        unsigned evt = 0;
                        toi_update(x, c, &evt);
                        if (x.record_events) put_update_events(x, wi, w, wd, evt, c);
                        if ((c.flags & kContactEnabled) == 0 || (c.flags & kContactTouching) == 0) {
                            b_set_sweep(O, backup);
                            b_sync_transform(O);
                            return true;
                        }
                        c.flags |= kContactIsland;
                        x.s_isl_contact[c0 + ncI++] = c0 + kk;
                        if (O.flags & kBodyIsland) return true;
                        O.flags |= kBodyIsland;
                        if (O.type != kStaticBody) b_set_awake(O, true);
                        x.s_isl_body[b0 + nbI++] = other;
                        return true;
                    };
                    if (Team::kLists) {
                        // the newer candidates first (higher positions), then the body's list
                        tm.scan_desc(ncand, touches, join, ncand0);
                        if (tm.lead()) {
                            for (int e = lstart[body], ee = lstart[body + 1]; e < ee; ++e)
                                if (!join(lent[e])) break;
                        }
                    } else {
                        tm.scan_desc(ncand, touches, join);
                    }
                }
                mark(4);
                nbI = tm.bcast(nbI);
                ncI = tm.bcast(ncI);
                if (rk < kWarp) solve_toi_island(x, w, wi, sb, nbI, ncI, mcb.x, mcb.y, (1.0f - minAlpha) * x.dt);
                tm.sync();
                int nnow = 0;
                if (tm.lead()) {
                    mark(5);
                    for (int i = 0; i < nbI; ++i) {
                        int body = x.s_isl_body[b0 + i];
                        dbox_body_state& Bd = x.bs[b0 + body];
                        Bd.flags &= ~(uint32_t)kBodyIsland;
                        if (Bd.type != kDynamicBody) continue;
                        x.s_bfl[b0 + body] = kBfMark;
                        sync_fixtures(x, b0 + body);
                        if (!big_toi) continue;
                        const BodyStatic& st = x.bst[b0 + body];                 // the proxies it moved
                        for (int e = 0; e < st.fix_count; ++e) {
                            const int r = x.body_fix[st.fix_start + e] - f0;
                            if (!x.px[f0 + r].moved || x.px[f0 + r].proxy_id < 0) continue;
                            pnow[nnow++] = r;
                            if (!toimv[r]) { toimv[r] = 1; pall[nall++] = r; }
                        }
                    }
                }
                nnow = tm.bcast(nnow);
                nall = tm.bcast(nall);
                nbI = tm.bcast(nbI);
                // invalidate the TOIs of every contact on a displaced dynamic body (only
                // candidates carry the two flags)
                if (Team::kLists) {
                    const int warp = rk >> 5, lane = rk & 31, nw = ts >> 5;
                    for (int i = warp; i < nbI; i += nw) {
                        const int body = x.s_isl_body[b0 + i];
                        if (!(x.s_bfl[b0 + body] & kBfMark)) continue;
                        for (int e = lstart[body] + lane, ee = lstart[body + 1]; e < ee; e += 32)
                            atomicAnd(&x.ct[c0 + cand[lent[e]]].flags, ~(uint32_t)(kContactToi | kContactIsland));
                    }
                }
                for (int t = (Team::kLists ? ncand0 : 0) + rk; t < ncand; t += ts) {
                    int k = cand[t];
                    int2 cb = x.s_cbody[c0 + k];
                    if ((x.s_bfl[b0 + cb.x] | x.s_bfl[b0 + cb.y]) & kBfMark) {
                        if (Team::kLists) atomicAnd(&x.ct[c0 + k].flags, ~(uint32_t)(kContactToi | kContactIsland));
                        else x.ct[c0 + k].flags &= ~(uint32_t)(kContactToi | kContactIsland);
                    }
                }
                tm.sync();
                for (int i = rk; i < nbI; i += ts) x.s_bfl[b0 + x.s_isl_body[b0 + i]] = 0;
                tm.sync();
                if (big_toi) {
                    const int total = nnow > 0 ? tm.first_warp([&]() { return toi_pairs_big(x, w, pnow, nnow, pall, nall, toimv); }) : 0;
                    if (total > 0) add_pairs_t(x, w, total, tm);
                } else {
                    tm.first_warp([&]() { find_new_contacts(x, w); return 0; });
                }
                ncand = tm.collect(n, wd.contact_count, cand, ncand, is_cand);
                tm.sync();
                mark(6);
            }
            advanced = true;
            if (solved && x.sub_stepping) {
                if (tm.lead()) wd.step_complete = 0;
                break;
            }
            if constexpr (Team::kLists) {
                // the next event's revisit list: the candidates of the bodies this event touched
                // (the new contacts' bodies included) and every candidate added since SolveTOI began
                ntb = tm.bcast(ntb);
                const int nnew = wd.contact_count - n;
                const bool over = ntb > nb || ntb + 2 * nnew > nb;
                if (!over)
                    for (int i = rk; i < nnew; i += ts) {
                        const int2 cb = x.s_cbody[c0 + n + i];
                        tbody[ntb + 2 * i] = cb.x;
                        tbody[ntb + 2 * i + 1] = cb.y;
                    }
                if (tm.lead()) tm.aux[2] = 0;
                tm.sync();
                if (!over) {
                    const int warp = rk >> 5, lane = rk & 31, nw = ts >> 5;
                    for (int i = warp; i < ntb + 2 * nnew; i += nw) {
                        const int bd = tbody[i];
                        if (x.bs[b0 + bd].type == kStaticBody) continue;
                        for (int e = lstart[bd] + lane, ee = lstart[bd + 1]; e < ee; e += 32) {
                            const int q = atomicAdd(&tm.aux[2], 1);
                            if (q < dcap) dset[q] = lent[e];
                        }
                    }
                    for (int t = ncand0 + rk; t < ncand; t += ts) {
                        const int q = atomicAdd(&tm.aux[2], 1);
                        if (q < dcap) dset[q] = t;
                    }
                }
                tm.sync();
                nd = tm.aux[2];
                full = over || nd > 1024 || nd > wi.contact_cap;
                tm.sync();
            }
        }
        if (tm.lead()) { wd.toi_events = events; wd.acc_toi_events += (unsigned long long)events; }
    }
    tm.sync();
    if (x.prof && tm.lead()) {
        unsigned long long* pr = x.prof + kProfSlots * (size_t)w;
        pr[16] = clock64() - t_start;
        pr[17] = wd.toi_events;
#pragma unroll
        for (int i = 0; i < 7; ++i) pr[18 + i] = tacc[i];
    }
    // b2World.Step epilogue (b2world.d:421-429)
    if (tm.lead() && x.dt > 0.0f) wd.inv_dt0 = x.inv_dt;
    if (wd.flags & 4u) {
        for (int i = rk; i < nb; i += ts) {
            dbox_body_state& B = x.bs[b0 + i];
            B.force[0] = 0.0f; B.force[1] = 0.0f; B.force[2] = 0.0f;
        }
    }
}

DG void toi_world(const Ctx& x, int w, float* sbp) { toi_world_t(x, w, sbp, WarpTeam()); }

// k_collide_finish for a large world on a block of kPairThreads threads: the same steps, the
// passes over its contacts spread over the block, the inactive contacts that a wake may
// revive handed to one thread in list order, and the stable compaction done as a prefix
// sum of destinations and a chunked in-place move (every destination is at or before its
// source, and a chunk is read completely before any of it is written)
__global__ void __launch_bounds__(kPairThreads) k_collide_finish_big(const __grid_constant__ Ctx x) {
    __shared__ int shi[32];
    __shared__ unsigned s_bal[32];
    __shared__ int s_box[2];
    __shared__ float s_ra[32];
    __shared__ int s_rl[32];
    __shared__ unsigned s_words[kPairThreads];
    __shared__ int s_aux[4];
    // on the world's cluster: every block a round-robin share of the passes over contacts and
    // bodies; the first block the revived contacts, the listener events and the scans
    const int csize = x.big_cluster > 1 ? (int)cluster_blocks() : 1;
    const int crank = csize > 1 ? (int)cluster_rank() : 0;
    const bool r0 = crank == 0;
    const int w = x.big_worlds[blockIdx.x / csize];
    const WorldInfo& wi = x.wi[w];
    WorldDyn& wd = x.wd[w];
    const int tid = threadIdx.x, nt = blockDim.x;
    const int gtid = tid * csize + crank, gsize = nt * csize;
    auto csync = [&]() { if (csize > 1) cluster_sync(); else __syncthreads(); };
    const int n = wd.contact_count, c0 = wi.contact_start;
    int* part = x.s_pcount + wi.fix_start;                               // per-block flags, per-chunk counts
    const long long t_in = clock64();
    BlockTeam tm{s_bal, s_box, s_ra, s_rl, s_words, s_aux};
    bool need = false;
    for (int k = gtid; k < n; k += gsize) {
        if (x.s_cstate[c0 + k] == 1) {
            const dbox_contact_state& c = x.ct[c0 + k];
            const int A = x.fx[c.fixture_a].body, B = x.fx[c.fixture_b].body;
            if (x.s_woken[A] != kNoWake || x.s_woken[B] != kNoWake) need = true;
        }
    }
    need = __syncthreads_or(need) != 0;
    if (csize > 1) {
        if (tid == 0) part[crank] = need ? 1 : 0;
        cluster_sync();
        need = false;
        for (int q = 0; q < csize; ++q) need |= ld_volatile_i(&part[q]) != 0;
        cluster_sync();                                                  // before `part` is reused
    }
    if (need && r0) {
        tm.scan_desc(n, [&](int k) { return x.s_cstate[c0 + k] == 1; }, [&](int k) {
            const int lp = n - 1 - k;
            dbox_contact_state& c = x.ct[c0 + k];
            const int A = x.fx[c.fixture_a].body, B = x.fx[c.fixture_b].body;
            const dbox_body_state& ba = x.bs[A];
            const dbox_body_state& bb = x.bs[B];
            const bool awA = (ba.flags & kBodyAwake) || x.s_woken[A] < lp;
            const bool awB = (bb.flags & kBodyAwake) || x.s_woken[B] < lp;
            const bool activeA = awA && ba.type != kStaticBody;
            const bool activeB = awB && bb.type != kStaticBody;
            if (!activeA && !activeB) return true;
            unsigned evt = 0;
            x.s_cstate[c0 + k] = collide_one(x, c, lp, false, &evt);
            if (x.record_events) x.s_cevt[c0 + k] = (unsigned char)evt;
            return true;
        });
    }
    // listener events of this Collide, in list order (newest contact first)
    if (x.record_events && r0) {
        __syncthreads();
        int base = 0;
        for (int top = n - 1; top >= 0; top -= nt) {
            const int k = top - tid;
            const unsigned evt = k >= 0 ? x.s_cevt[c0 + k] : 0u;
            int all;
            int slot = base + block_scan_value(__popc(evt), shi, &all);
            if (evt) {
                const dbox_contact_state& c = x.ct[c0 + k];
                if (evt & 1u) put_event(x, wi, w, slot++, DBOX_EVENT_BEGIN, c, c.point_count, nullptr, nullptr);
                if (evt & 2u) put_event(x, wi, w, slot++, DBOX_EVENT_END, c, c.point_count, nullptr, nullptr);
                if (evt & 4u) put_event(x, wi, w, slot++, DBOX_EVENT_PRESOLVE, c, c.point_count, nullptr, nullptr);
            }
            base += all;
        }
        if (tid == 0) wd.ev_count = base;
    }
    csync();
    // apply wakes
    for (int i = gtid; i < wi.body_count; i += gsize) {
        const int b = wi.body_start + i;
        if (x.s_woken[b] != kNoWake) b_set_awake(x.bs[b], true);
    }
    // stable compaction of surviving contacts: kept contacts per chunk of nt, the chunks'
    // offsets (first block), each contact's destination, then the move
    int* dst = x.s_tcand + c0;
    const int nch = (n + nt - 1) / nt;
    for (int c = crank; c < nch; c += csize) {
        const int k = c * nt + tid;
        int all;
        block_scan_value(k < n && x.s_cstate[c0 + k] != 2 ? 1 : 0, shi, &all);
        if (tid == 0) part[c] = all;
    }
    if (r0 && tid == 0) part[nch] = 0;
    csync();
    if (r0) block_exclusive_scan(part, nch + 1, shi);
    csync();
    const int out = ld_volatile_i(&part[nch]);
    for (int c = crank; c < nch; c += csize) {
        const int k = c * nt + tid;
        const int keep = k < n && x.s_cstate[c0 + k] != 2;
        int all;
        const int d = ld_volatile_i(&part[c]) + block_scan_value(keep, shi, &all);
        if (k < n) dst[k] = keep ? d : -1;
    }
    csync();
    if (out < n) {
        // every destination is at or before its source, so the blocks move csize chunks at a
        // time: all of them read their chunk, then all of them write it
        constexpr int kWords = (int)(sizeof(dbox_contact_state) / sizeof(int4));
        static_assert(sizeof(dbox_contact_state) % sizeof(int4) == 0, "contacts move as 16-byte words");
        int4* words = reinterpret_cast<int4*>(x.ct + c0);
        const int chunk = 4 * nt / kWords;                               // contacts a block reads at once
        for (int wave = 0; wave * chunk * csize < n; ++wave) {
            const int base = (wave * csize + crank) * chunk;
            const int cnt = base >= n ? 0 : (n - base < chunk ? n - base : chunk);
            int4 v[4];
            int to[4];
#pragma unroll
            for (int j = 0; j < 4; ++j) {
                const int q = tid + j * nt;                              // word of this chunk
                to[j] = -1;
                if (q < cnt * kWords) {
                    const int k = base + q / kWords;
                    const int dk = dst[k];
                    if (dk >= 0 && dk != k) {
                        to[j] = dk * kWords + q % kWords;
                        v[j] = words[(size_t)base * kWords + q];
                    }
                }
            }
            csync();
#pragma unroll
            for (int j = 0; j < 4; ++j)
                if (to[j] >= 0) words[to[j]] = v[j];
            csync();
        }
    }
    if (r0 && tid == 0) { wd.contact_count = out; wd.acc_contacts += (unsigned long long)n; wd.acc_steps += 1; }
    if (r0 && x.prof && tid == 0) x.prof[kProfSlots * (size_t)w + 15] = clock64() - t_in;
}


// The passes at the start of a large world's SolveTOI (b2world.d:1131-1146, and the candidate
// filter of :1172-1188) on its cluster, each block a round-robin share: every body's island
// flag and alpha0 cleared, every contact compacted and its TOI state cleared, the candidates
// marked in one ballot word per 32 contact slots; then the first block lists the candidates in
// slot order from the words while every block counts each dynamic body's candidates, a scan
// of the counts (each block a contiguous range of bodies, then the ranges' offsets), the lists
// filled with candidate positions and each list sorted by descending position.  The same lists
// as the single-block passes in toi_world_t (a list's order comes from its sort alone).
DG void toi_begin_cluster(const Ctx& x, int w, int csize, int crank, int* shi) {
    const WorldInfo& wi = x.wi[w];
    WorldDyn& wd = x.wd[w];
    if (!(x.continuous && x.dt > 0.0f)) return;                          // no SolveTOI
    const int tid = threadIdx.x, nt = blockDim.x, lane = lane_id();
    const int gtid = tid * csize + crank, gsize = nt * csize;
    const int gwarp = (tid >> 5) * csize + crank, gnw = (nt >> 5) * csize;
    auto csync = [&]() { if (csize > 1) cluster_sync(); else __syncthreads(); };
    const int b0 = wi.body_start, nb = wi.body_count, c0 = wi.contact_start, f0 = wi.fix_start;
    const int n = ld_volatile_i(&wd.contact_count);                     // after AddPair
    const bool clear = wd.step_complete != 0;
    const bool big_toi = wi.pair_block && wd.g_valid && !wi.proxy_order;
    int* cand = x.s_tcand + c0;
    unsigned* words = reinterpret_cast<unsigned*>(x.s_cstate + c0);     // candidate bits per 32 slots
    int* lstart = x.s_adj_start + wi.bx_start;                          // nb + 1
    int* lcur = x.s_cursor + b0;
    int* lent = reinterpret_cast<int*>(x.s_adj_items + 2 * (size_t)c0);
    int* part = x.s_pcount + f0;                                         // per block: its range's total
    auto dyn = [&](int b) { return x.bs[b0 + b].type != kStaticBody; };
    for (int i = gtid; i < nb; i += gsize) {
        if (clear) {
            x.bs[b0 + i].flags &= ~(uint32_t)kBodyIsland;
            x.bs[b0 + i].sweep[8] = 0.0f;
        }
        x.s_bfl[b0 + i] = 0;
        lstart[i] = 0;
    }
    if (big_toi)
        for (int i = gtid; i < wi.fix_count; i += gsize) x.s_sapk[0][f0 + i] = 0;   // moved during this SolveTOI
    const int nwd = (n + 31) >> 5;
    for (int q = gwarp; q < nwd; q += gnw) {
        const int k = 32 * q + lane;
        bool hit = false;
        if (k < n) {
            contact_compact(x, c0 + k, b0);
            if (clear) {
                dbox_contact_state& c = x.ct[c0 + k];
                c.flags &= ~(uint32_t)(kContactToi | kContactIsland);
                c.toi_count = 0;
                c.toi = 1.0f;
            }
            hit = toi_candidate(x, c0 + k, b0);
        }
        const unsigned bal = __ballot_sync(0xffffffffu, hit);
        if (lane == 0) words[q] = bal;
    }
    csync();
    for (int q = gwarp; q < nwd; q += gnw) {                             // candidates per dynamic body
        if (!((words[q] >> lane) & 1u)) continue;
        const int2 cb = x.s_cbody[c0 + 32 * q + lane];
        if (dyn(cb.x)) atomicAdd(&lstart[cb.x], 1);
        if (dyn(cb.y)) atomicAdd(&lstart[cb.y], 1);
    }
    if (crank == 0) {                                                    // the candidate list
        int cnt = 0;
        for (int base = 0; base < nwd; base += nt) {
            const int q = base + tid;
            const unsigned m = q < nwd ? words[q] : 0u;
            int all;
            int pos = cnt + block_scan_value(__popc(m), shi, &all);
            for (unsigned b = m; b; b &= b - 1u) cand[pos++] = 32 * q + __ffs(b) - 1;
            cnt += all;
        }
        if (tid == 0) wd.toi_ncand = cnt;
    }
    csync();
    const int chunk = (nb + csize - 1) / csize;                          // this block's bodies
    const int lo = min(nb, crank * chunk), hi = min(nb, lo + chunk);
    const int tot = block_exclusive_scan(lstart + lo, hi - lo, shi);
    if (tid == 0) part[crank] = tot;
    csync();
    int off = 0, all = 0;
    for (int r = 0; r < csize; ++r) {
        const int v = ld_volatile_i(&part[r]);
        off += r < crank ? v : 0;
        all += v;
    }
    for (int i = lo + tid; i < hi; i += nt) {
        const int v = lstart[i] + off;
        lstart[i] = v;
        lcur[i] = v;
    }
    if (crank == 0 && tid == 0) lstart[nb] = all;
    csync();
    const int ncand = ld_volatile_i(&wd.toi_ncand);
    for (int t = gtid; t < ncand; t += gsize) {
        const int2 cb = x.s_cbody[c0 + cand[t]];
        if (dyn(cb.x)) lent[atomicAdd(&lcur[cb.x], 1)] = t;
        if (dyn(cb.y)) lent[atomicAdd(&lcur[cb.y], 1)] = t;
    }
    csync();
    for (int i = gtid; i < nb; i += gsize) {                             // each list by descending position
        const int e0 = lstart[i], d = lstart[i + 1] - e0;
        int gap = 1;
        while (3 * gap + 1 < d) gap = 3 * gap + 1;
        for (; gap > 0; gap /= 3)
            for (int a = e0 + gap; a < e0 + d; ++a) {
                const int v = lent[a];
                int q = a - gap;
                while (q >= e0 && lent[q] < v) { lent[q + gap] = lent[q]; q -= gap; }
                lent[q + gap] = v;
            }
    }
}

// AddPair for a large world's pairs on its cluster, then the passes at the start of its SolveTOI
__global__ void __launch_bounds__(kPairThreads) k_finish_big_block(const __grid_constant__ Ctx x) {
    __shared__ int s_rl[32];
    const int csize = x.big_cluster > 1 ? (int)cluster_blocks() : 1;
    const int crank = csize > 1 ? (int)cluster_rank() : 0;
    const int w = x.big_worlds[blockIdx.x / csize];
    const int total = x.wd[w].pair_total;
    const long long t_in = clock64();
    if (total > 0) add_pairs_cluster(x, w, total, csize, crank, s_rl);   // the same decision in every block
    const long long t_add = clock64();
    if (csize > 1) cluster_sync();                                       // the contact count and new contacts
    toi_begin_cluster(x, w, csize, crank, s_rl);
    if (x.prof && crank == 0 && threadIdx.x == 0) {
        x.prof[kProfSlots * (size_t)w + 31] = t_add - t_in;
        x.prof[kProfSlots * (size_t)w + 29] = clock64() - t_add;
    }
}

// A large world's SolveTOI event loop on a block of its own: kToiThreads threads, so that the
// serial parts (the lead's event contact, the sub-step solve, the TOI computations) keep their
// values in registers
constexpr int kToiThreads = 512;
__global__ void __launch_bounds__(kToiThreads, 1) k_toi_big(const __grid_constant__ Ctx x) {
    __shared__ unsigned s_bal[32];
    __shared__ int s_box[2];
    __shared__ float s_ra[32];
    __shared__ int s_rl[32];
    __shared__ unsigned s_words[kToiThreads];
    __shared__ int s_aux[4];
    const int w = x.big_worlds[blockIdx.x];
    BlockTeam tm{s_bal, s_box, s_ra, s_rl, s_words, s_aux};
    toi_world_t(x, w, x.s_sbody + 6 * (size_t)x.wi[w].body_start, tm, true);
}

// ------------------------------------------------------------ b2World.Solve of a large world on a cluster
// A world of 4,096+ fixtures is one warp's dependent walk in solve_world; here a thread-block
// cluster (k_solve_big, up to 8 blocks of kBigThreads threads) does the same step: the same
// islands in the same order, the same constraint order inside each island, the same
// arithmetic, so the same bits.  The first block runs the serial phases:
//   islands: the island graph's components (contacts that are enabled, touching and not a
//     sensor, joints between active bodies; static bodies do not connect) by a lock-free
//     union-find; the reference's depth-first search (b2world.d:959-1095) seeds islands in body
//     list order (descending index), so an island's seed is the highest-index awake, active,
//     non-static body of its component and islands are numbered by descending seed; a prefix sum
//     of the components' body / contact / joint counts places each island's lists, and each
//     island's own search (the reference's, from its seed) runs on a thread of its own.  A
//     static body is never pushed: popping one changes nothing but its island mark, which is the
//     last island (in order) that reached it.
//   schedules: each island's constraints get their levels on one thread (islands share no
//     dynamic body), then the block buckets all constraints by level.
// Every block runs the parallel phases, items dealt round-robin over the cluster's threads:
// compaction, integration, constraint rows, the sweeps (levels in order, a level's rows over
// the cluster, a cluster barrier between levels), StoreImpulses, copy back and sleep.
// Every warm-start mode runs here too: the predictions of mode 2 on kInferWarps warps of the
// first block, 16 rows a pass.
constexpr int kBigThreads = 1024;
constexpr int kInferWarps = 8;
constexpr int kInferStage = 16 * kFeat + 2 * 16 * kHid;               // bf16 per warp: X, H1, H2
constexpr int kBigSmemInfer = kInferWarps * kInferStage * 2;          // bytes

DG int uf_find(int* parent, int i) {
    // parents only ever point to lower indices, so the walk ends; path halving
    for (;;) {
        const int p = ld_volatile_i(&parent[i]);
        if (p == i) return i;
        const int g = ld_volatile_i(&parent[p]);
        if (g != p) parent[i] = g;
        i = p;
    }
}
DG void uf_union(int* parent, int a, int b) {
    for (;;) {
        a = uf_find(parent, a);
        b = uf_find(parent, b);
        if (a == b) return;
        if (a < b) { const int t = a; a = b; b = t; }                     // the larger root under the smaller
        if (atomicCAS(&parent[a], a, b) == a) return;
    }
}

// ---- the level sweeps of a large world's Solve, spread over a thread-block cluster

// What a row of a sweep needs (the same for every block of the cluster)
struct BigSweep {
    int b0, kx;
    VRow* vrow;
    PRow* prow;
    SB sb;
    bool warm;
    float dtRatio;
    int njI, maxLv, maxLp;
    const int* lvl_v;
    const int* lvl_p;
    const int* sched_p;
    int* iflags;
    unsigned* iminsep;
};
// warm start of a contact, or a joint's InitVelocityConstraints (b2island.d:133-146)
DG void big_warm_row(const Ctx& x, const BigSweep& s, int idx) {
    if (s.njI == 0) { warm_start(unpack_v(load_v(s.vrow + idx)), s.sb); return; }
    const int item = s.sched_p[s.kx + idx];
    if (item >= 0) { if (s.warm) warm_start(unpack_v(load_v(s.vrow + x.s_vpos[item])), s.sb); }
    else joint_init(x, -item - 1, s.b0, s.sb, s.warm, s.dtRatio);
}
// one row of a velocity iteration (b2contactsolver.d:492-772, the joints' SolveVelocityConstraints)
DG void big_vel_row(const Ctx& x, const BigSweep& s, int idx, int it) {
    const VRow r = load_v(s.vrow + idx);
    if (r.ids.w >= 0) {
        if (it == 0 && (r.ids.z & 0x100)) {                          // a predicted start (ws mode 2)
            float4 im;
            solve_velocity_learned(r, s.sb, &im);
            s.vrow[idx].imp = im;
            return;
        }
        VC vc = unpack_v(r);
        BodyVel q = load_vel(s.sb, vc.bodyA, vc.bodyB);
        if (vc.pointCount == 2) solve_velocity_two(vc, q);
        else solve_velocity(vc, q);
        store_vel(s.sb, vc.bodyA, vc.bodyB, q);
        s.vrow[idx].imp = make_float4(vc.p[0].normalImpulse, vc.p[0].tangentImpulse, vc.p[1].normalImpulse,
                                      vc.p[1].tangentImpulse);
    } else {
        joint_solve_velocity(x, -r.ids.w - 1, s.b0, s.sb);
    }
}
// one row of a position iteration, skipping islands already solved (b2island.d:206-224)
DG void big_pos_row(const Ctx& x, const BigSweep& s, int idx) {
    const PRow r = load_p(s.prow + idx);
    const int is = r.ids.w;
    if (s.iflags[is] & 1) return;
    if (r.ids.z >= 0) {
        const float ms = solve_position_row(unpack_p(r), s.sb);
        atomicMin(&s.iminsep[is], fkey(ms));
    } else if (!joint_solve_position(x, -r.ids.z - 1, s.b0, s.sb)) {
        atomicOr(&s.iflags[is], 4);
    }
}
// levels 1..maxL in order with a barrier between levels.  On a cluster, a level of more than
// kNarrowRows rows is dealt over the cluster's threads and ends in a cluster barrier; a run of
// narrower levels is swept by the first block alone (r0), with block barriers between its
// levels, while the other blocks wait at the cluster barrier after the run: a cluster barrier
// costs thousands of cycles however few the level's rows.  Rows and body state live in global
// memory, so any block may sweep any level; every block finds the same runs.
constexpr int kNarrowRows = 128;
template <class F>
DG void cluster_levels(const int* lvl, int maxL, int gtid, int gsize, bool clustered, bool r0, F&& f) {
    const int tid = threadIdx.x, nt = blockDim.x;
    for (int L = 1; L <= maxL;) {
        const int s = lvl[L], e = lvl[L + 1];
        const bool wide = !clustered || e - s > kNarrowRows;
        if (!wide && !r0) {                                             // a run of narrow levels: wait after it
            while (L <= maxL && lvl[L + 1] - lvl[L] <= kNarrowRows) ++L;
            cluster_sync();
            continue;
        }
        for (int idx = wide ? s + gtid : s + tid; idx < e; idx += wide ? gsize : nt) f(idx);   // one call site
        ++L;
        if (!clustered) __syncthreads();
        else if (wide || L > maxL || lvl[L + 1] - lvl[L] > kNarrowRows) cluster_sync();   // the cluster meets
        else __syncthreads();                                           // the first block's next narrow level
    }
}
__global__ void __launch_bounds__(kBigThreads) k_solve_big(const __grid_constant__ Ctx x) {
    extern __shared__ __align__(16) float big_smem[];                  // ws mode 2: the inference staging
    __shared__ int shi[32];
    __shared__ float shf[32];
    __shared__ int s_next, s_maxv, s_maxp;
    const int csize = x.big_cluster > 1 ? (int)cluster_blocks() : 1;
    const int crank = csize > 1 ? (int)cluster_rank() : 0;
    const bool clustered = csize > 1;
    const int w = x.big_worlds[blockIdx.x / csize];
    const WorldInfo& wi = x.wi[w];
    WorldDyn& wd = x.wd[w];
    const int tid = threadIdx.x, nt = blockDim.x;
    if (!(wd.step_complete && x.dt > 0.0f)) return;                    // the same decision in every block
    // the first block (r0) runs the serial phases; the parallel ones are dealt round-robin over
    // the cluster's threads, a cluster barrier (a block barrier without a cluster) between phases
    const bool r0 = crank == 0;
    const int gtid = tid * csize + crank, gsize = nt * csize;
    auto csync = [&]() { if (clustered) cluster_sync(); else __syncthreads(); };
    if (r0 && x.prof && tid == 0) {
        unsigned smid;
        asm volatile("mov.u32 %0, %%smid;" : "=r"(smid));
        x.prof[kProfSlots * (size_t)w + 27] = csize;
        x.prof[kProfSlots * (size_t)w + 28] = smid;
    }
    const int b0 = wi.body_start, nb = wi.body_count;
    const int c0 = wi.contact_start, n = wd.contact_count;
    const int j0 = wi.joint_start, nj = wi.joint_count;
    const int bx = wi.bx_start, kx = wi.kx_start;
    const float h = x.dt;
    const bool warm = x.warm_starting != 0;
    const float dtRatio = wd.inv_dt0 * x.dt;                            // b2world.d:392
    auto stampb = [&](int slot) { if (r0 && x.prof && tid == 0) x.prof[kProfSlots * (size_t)w + slot] = clock64(); };
    stampb(0);
    if (r0 && x.measure && tid == 0) { wd.q_sumsq = 0.0f; wd.q_max = 0.0f; wd.q_points = 0; wd.q_minsep = 0.0f; }
    SB sb;
    sb.p = x.s_sbody + 6 * (size_t)b0;
    int* iflags = x.s_isl_flags + b0;
    unsigned* iminsep = x.s_isl_minsep + b0;
    unsigned char* bfl = x.s_bfl + b0;
    int* body_island = x.s_body_island + b0;
    int* adj = x.s_adj_start + bx;                                       // nb + 1
    int* isl_body = x.s_isl_body + b0;
    int* isl_contact = x.s_isl_contact + c0;
    int2* isl_pair = x.s_isl_pair + c0;
    int* isl_joint = x.s_isl_joint + j0;
    unsigned char* cvis = x.s_cvis + c0;
    int2* items = x.s_adj_items + 2 * (size_t)c0;
    // compact per-body / per-contact data; island flags cleared (b2world.d:944-957)
    for (int i = gtid; i < nb; i += gsize) {
        dbox_body_state& B = x.bs[b0 + i];
        B.flags &= ~(uint32_t)kBodyIsland;
        bfl[i] = body_flag_byte(B);
        body_island[i] = -1;
        sb_load(sb, i, B);
        adj[i] = 0;
    }
    for (int k = gtid; k < n; k += gsize) {
        x.ct[c0 + k].flags &= ~(uint32_t)kContactIsland;
        contact_compact(x, c0 + k, b0);
        cvis[k] = 0;
    }
    for (int j = gtid; j < nj; j += gsize) x.jt[j0 + j].island_flag = 0;
    csync();
    int nIsl = 0, nbI = 0, ncI = 0, njI = 0, maxLv = 0, maxLp = 0, nItems = 0;
    if (r0) {
    // contact edges of the island graph per body, newest contact first (b2world.d:1026-1062);
    // a static body's list is never walked (the search does not continue through it), so
    // it gets none
    for (int k = tid; k < n; k += nt) {
        if (x.s_cq[c0 + k] & 1) {
            const int2 cb = x.s_cbody[c0 + k];
            if (!(bfl[cb.x] & kBfStatic)) atomicAdd(&adj[cb.x], 1);
            if (!(bfl[cb.y] & kBfStatic)) atomicAdd(&adj[cb.y], 1);
        }
    }
    __syncthreads();
    {
        const int tot = block_exclusive_scan(adj, nb, shi);
        if (tid == 0) adj[nb] = tot;
    }
    int* cursor = x.s_cursor + b0;
    for (int i = tid; i < nb; i += nt) cursor[i] = adj[i];
    __syncthreads();
    for (int k = tid; k < n; k += nt) {
        if (x.s_cq[c0 + k] & 1) {
            const int2 cb = x.s_cbody[c0 + k];
            if (!(bfl[cb.x] & kBfStatic)) items[atomicAdd(&cursor[cb.x], 1)] = make_int2(k, cb.y);
            if (!(bfl[cb.y] & kBfStatic)) items[atomicAdd(&cursor[cb.y], 1)] = make_int2(k, cb.x);
        }
    }
    __syncthreads();
    for (int i = tid; i < nb; i += nt) {                                 // each list by descending contact
        const int e0 = adj[i], d = adj[i + 1] - e0;
        int gap = 1;                                                     // Shell sort, gaps 1, 4, 13, 40, ...
        while (3 * gap + 1 < d) gap = 3 * gap + 1;
        for (; gap > 0; gap /= 3)
            for (int a = e0 + gap; a < e0 + d; ++a) {
                const int2 v = items[a];
                int b = a - gap;
                while (b >= e0 && items[b].x < v.x) { items[b + gap] = items[b]; b -= gap; }
                items[b + gap] = v;
            }
    }
    __syncthreads();
    stampb(1);
    // ---- islands: components, seeds, order, sizes
    int* parent = x.s_stack + b0;
    int* root = x.s_cursor + b0;
    int* seedmax = x.s_last + b0;
    int* rid = x.s_woken + b0;                                           // island of a component root
    int* seedf = reinterpret_cast<int*>(x.s_isl_sleep + b0);
    int* seed_of = reinterpret_cast<int*>(x.s_isl_minsep + b0);
    int* cntb = x.s_isl_bstart + bx;
    int* cntc = x.s_isl_cstart + bx;
    int* cntj = x.s_isl_jstart + bx;
    auto nonstatic = [&](int i) { return (bfl[i] & kBfStatic) == 0; };
    auto active = [&](int i) { return (bfl[i] & kBfActive) != 0; };
    for (int i = tid; i < nb; i += nt) { parent[i] = i; seedmax[i] = -1; rid[i] = -1; }
    __syncthreads();
    for (int k = tid; k < n; k += nt) {
        if (!(x.s_cq[c0 + k] & 1)) continue;
        const int2 cb = x.s_cbody[c0 + k];
        if (nonstatic(cb.x) && nonstatic(cb.y)) uf_union(parent, cb.x, cb.y);
    }
    for (int j = tid; j < nj; j += nt) {
        const DJoint& jj = x.jt[j0 + j];
        if (jj.type < 0) continue;
        const int A = jj.body_a - b0, B = jj.body_b - b0;
        if (nonstatic(A) && nonstatic(B) && active(A) && active(B)) uf_union(parent, A, B);
    }
    __syncthreads();
    for (int i = tid; i < nb; i += nt) {
        const int r = uf_find(parent, i);
        root[i] = r;
        const unsigned char f = bfl[i];
        if ((f & kBfAwake) && (f & kBfActive) && !(f & kBfStatic)) atomicMax(&seedmax[r], i);
    }
    __syncthreads();
    for (int i = tid; i < nb; i += nt) {                                 // islands by descending seed
        const int d = nb - 1 - i;
        seedf[i] = seedmax[root[d]] == d ? 1 : 0;
    }
    __syncthreads();
    nIsl = block_exclusive_scan(seedf, nb, shi);
    for (int i = tid; i < nb; i += nt) {
        const int d = nb - 1 - i;
        if (seedmax[root[d]] == d) { rid[root[d]] = seedf[i]; seed_of[seedf[i]] = d; }
    }
    for (int k = tid; k <= nIsl; k += nt) { cntb[k] = 0; cntc[k] = 0; cntj[k] = 0; }
    __syncthreads();
    for (int i = tid; i < nb; i += nt)
        if (nonstatic(i) && rid[root[i]] >= 0) atomicAdd(&cntb[rid[root[i]]], 1);
    for (int k = tid; k < n; k += nt) {
        if (!(x.s_cq[c0 + k] & 1)) continue;
        const int2 cb = x.s_cbody[c0 + k];
        const int d = nonstatic(cb.x) ? cb.x : cb.y;
        if (rid[root[d]] >= 0) atomicAdd(&cntc[rid[root[d]]], 1);
    }
    for (int j = tid; j < nj; j += nt) {
        const DJoint& jj = x.jt[j0 + j];
        if (jj.type < 0) continue;
        const int A = jj.body_a - b0, B = jj.body_b - b0;
        if (!active(A) || !active(B)) continue;
        const int d = nonstatic(A) ? A : (nonstatic(B) ? B : -1);
        if (d >= 0 && rid[root[d]] >= 0) atomicAdd(&cntj[rid[root[d]]], 1);
    }
    __syncthreads();
    nbI = block_exclusive_scan(cntb, nIsl, shi);
    ncI = block_exclusive_scan(cntc, nIsl, shi);
    njI = block_exclusive_scan(cntj, nIsl, shi);
    if (tid == 0) { cntb[nIsl] = nbI; cntc[nIsl] = ncI; cntj[nIsl] = njI; wd.islands = nIsl; s_next = 0; }
    __syncthreads();
    if (tid == 0) wd.sw_nisl = nIsl;
    }                                                                    // r0
    csync();
    if (!r0) nIsl = ld_volatile_i(&wd.sw_nisl);
    // ---- each island's depth-first search (b2world.d:988-1076), an island per thread, the
    // islands dealt round-robin over the cluster's blocks (they share no non-static body,
    // contact or joint; spread over the blocks, the searches' scattered loads and stores are
    // spread over as many SMs' load/store units)
    {
    int* parent = x.s_stack + b0;
    const int* seed_of = reinterpret_cast<const int*>(x.s_isl_minsep + b0);
    const int* cntb = x.s_isl_bstart + bx;
    const int* cntc = x.s_isl_cstart + bx;
    const int* cntj = x.s_isl_jstart + bx;
    for (int k = crank + csize * tid; k < nIsl; k += csize * nt) {
        const int seed = seed_of[k];
        int* stack = parent + cntb[k];                                   // this island's own stack rows
        int nB = cntb[k], nC = cntc[k], nJ = cntj[k];
        int top = 0;
        stack[top++] = seed;
        bfl[seed] |= kBfVisited;
        while (top > 0) {
            const int b = stack[--top];
            body_island[b] = k;
            isl_body[nB++] = b;
            bfl[b] |= kBfPopped;
            for (int e = adj[b], ee = adj[b + 1]; e < ee; ++e) {
                const int2 it = items[e];
                // the contact is in an island already exactly when its other body is non-static
                // and was popped before (its walk added it): one load instead of the contact's mark
                const unsigned char fo = bfl[it.y];
                if ((fo & (kBfPopped | kBfStatic)) == kBfPopped) continue;
                isl_contact[nC] = c0 + it.x;
                isl_pair[nC] = make_int2(b, it.y);
                ++nC;
                cvis[it.x] = 1;
                if (fo & kBfStatic) { atomicMax(&body_island[it.y], k); continue; }
                if (fo & kBfVisited) continue;
                stack[top++] = it.y;
                bfl[it.y] = fo | kBfVisited;
            }
            if (nj == 0) continue;
            const BodyStatic& st = x.bst[b0 + b];
            for (int e = 0; e < st.jadj_count; ++e) {
                const int j = x.jadj_joint[st.jadj_start + e];
                if (x.jt[j].island_flag) continue;
                const int other = x.jadj_other[st.jadj_start + e] - b0;
                const unsigned char fo = bfl[other];
                if ((fo & kBfActive) == 0) continue;
                isl_joint[nJ++] = j;
                x.jt[j].island_flag = 1;
                if (fo & kBfStatic) { atomicMax(&body_island[other], k); continue; }
                if (fo & kBfVisited) continue;
                stack[top++] = other;
                bfl[other] = fo | kBfVisited;
            }
        }
    }
    }
    csync();
    if (r0) {
    __syncthreads();
    stampb(2);
    for (int k = tid; k < n; k += nt)
        if (cvis[k]) x.ct[c0 + k].flags |= kContactIsland;
    // ---- level schedules: each island's walk on one lane, then the block buckets by level
    int* last = x.s_last + b0;
    for (int i = tid; i < nb; i += nt) last[i] = 0;
    if (tid == 0) { s_maxv = 0; s_maxp = 0; }
    __syncthreads();
    auto walk = [&](int k, bool contacts_first, int* maxl) {           // one lane: island k
        int ml = 0;
        for (int pass = 0; pass < 2; ++pass) {
            const bool doContacts = (pass == 0) == contacts_first;
            const int t0 = doContacts ? x.s_isl_cstart[bx + k] : x.s_isl_jstart[bx + k];
            const int t1 = doContacts ? x.s_isl_cstart[bx + k + 1] : x.s_isl_jstart[bx + k + 1];
            // the position of the walk in the all-contacts-then-all-joints order of build_schedule
            const int at = doContacts ? (contacts_first ? 0 : njI) : (contacts_first ? ncI : 0);
            for (int t = t0; t < t1; ++t) {
                int item, A, B, C = -1, D = -1;
                if (doContacts) {
                    item = isl_contact[t];
                    const int2 pr = isl_pair[t];
                    A = pr.x;
                    B = pr.y;
                } else {
                    item = -(isl_joint[t] + 1);
                    item_bodies(x, item, b0, A, B);
                    const DJoint& jj = x.jt[-item - 1];
                    if (jj.type == kGearJoint) { C = jj.body_c - b0; D = jj.body_d - b0; }
                }
                const bool dA = (bfl[A] & kBfDynamic) != 0, dB = (bfl[B] & kBfDynamic) != 0;
                int l = bmax(dA ? last[A] : 0, dB ? last[B] : 0);
                const bool dC = C >= 0 && (bfl[C] & kBfDynamic) != 0, dD = D >= 0 && (bfl[D] & kBfDynamic) != 0;
                if (dC && last[C] > l) l = last[C];
                if (dD && last[D] > l) l = last[D];
                l += 1;
                if (dA) last[A] = l;
                if (dB) last[B] = l;
                if (dC) last[C] = l;
                if (dD) last[D] = l;
                ml = l > ml ? l : ml;
                x.s_level[kx + at + t] = l;
                x.s_tmp[kx + at + t] = item;
            }
        }
        atomicMax(maxl, ml);
    };
    nItems = ncI + njI;
    auto bucket = [&](int maxL, int* sched, int* lvl) {
        for (int l = tid; l <= maxL + 1; l += nt) lvl[kx + l] = 0;
        __syncthreads();
        for (int i = tid; i < nItems; i += nt) atomicAdd(&lvl[kx + x.s_level[kx + i]], 1);
        __syncthreads();
        block_exclusive_scan(lvl + kx, maxL + 2, shi);
        for (int l = tid; l <= maxL + 1; l += nt) x.s_lcur[kx + l] = lvl[kx + l];
        __syncthreads();
        for (int i = tid; i < nItems; i += nt) {
            const int pos = atomicAdd(&x.s_lcur[kx + x.s_level[kx + i]], 1);
            sched[kx + pos] = x.s_tmp[kx + i];
        }
        __syncthreads();
    };
    for (int k = tid; k < nIsl; k += nt) walk(k, false, &s_maxv);
    __syncthreads();
    maxLv = s_maxv;
    bucket(maxLv, x.s_sched_v, x.s_lvl_v);
    maxLp = maxLv;
    if (njI) {
        for (int i = tid; i < nb; i += nt) last[i] = 0;
        __syncthreads();
        for (int k = tid; k < nIsl; k += nt) walk(k, true, &s_maxp);
        __syncthreads();
        maxLp = s_maxp;
        bucket(maxLp, x.s_sched_p, x.s_lvl_p);
    }
    if (x.prof && tid == 0) { x.prof[kProfSlots * (size_t)w + 12] = maxLv; x.prof[kProfSlots * (size_t)w + 13] = n; x.prof[kProfSlots * (size_t)w + 14] = nb; }
    stampb(3);
    if (tid == 0) {
        wd.acc_isl_bodies += (unsigned long long)nbI;
        wd.acc_isl_contacts += (unsigned long long)ncI;
        wd.acc_vsolve += (unsigned long long)ncI * (unsigned long long)x.vel_iters;
        // what the other blocks of the cluster need
        wd.sw_maxv = maxLv; wd.sw_maxp = maxLp; wd.sw_njI = njI;
        wd.sw_nisl = nIsl; wd.sw_nbi = nbI; wd.sw_nci = ncI; wd.sw_npend = 0;
    }
    }                                                                    // r0
    csync();
    if (!r0) {
        maxLv = ld_volatile_i(&wd.sw_maxv);
        maxLp = ld_volatile_i(&wd.sw_maxp);
        njI = ld_volatile_i(&wd.sw_njI);
        nIsl = ld_volatile_i(&wd.sw_nisl);
        nbI = ld_volatile_i(&wd.sw_nbi);
        ncI = ld_volatile_i(&wd.sw_nci);
        nItems = ncI + njI;
    }
    int* sched_p = njI ? x.s_sched_p : x.s_sched_v;
    int* lvl_p = njI ? x.s_lvl_p : x.s_lvl_v;
    // island flags and SetAwake(true) of the search (b2world.d:985-1004), applied after it
    for (int i = gtid; i < nb; i += gsize) {
        dbox_body_state& B = x.bs[b0 + i];
        if ((bfl[i] & kBfVisited) && !(bfl[i] & kBfStatic)) B.flags |= kBodyIsland;
        if (body_island[i] >= 0) b_set_awake(B, true);
    }
    // integrate velocities (b2island.d:82-116)
    for (int t = gtid; t < nbI; t += gsize) {
        const int i = isl_body[t];
        dbox_body_state& B = x.bs[b0 + i];
        B.sweep[2] = B.sweep[4];
        B.sweep[3] = B.sweep[5];
        B.sweep[6] = B.sweep[7];
        if (B.type == kDynamicBody) {
            const BodyStatic& st = x.bst[b0 + i];
            float2 v = sb.v(i);
            float wv = sb.w(i);
            float2 g = st.gravity_scale * x.gravity + B.mass[1] * v2(B.force[0], B.force[1]);
            v += h * g;
            wv += (h * B.mass[3]) * B.force[2];
            v *= fdiv(1.0f, 1.0f + h * st.lin_damping);
            wv *= fdiv(1.0f, 1.0f + h * st.ang_damping);
            sb.set_v(i, v, wv);
        }
    }
    csync();
    // constraint rows in schedule order (b2contactsolver.d:244-450), with the warm-start modes'
    // part of each contact row; rows waiting for a prediction listed in s_pend
    VRow* vrow = x.vr + kx;
    PRow* prow = x.pr + kx;
    for (int idx = gtid; idx < nItems; idx += gsize) {
        const int item = x.s_sched_v[kx + idx];
        bool pdone = false;
        if (item >= 0) {
            VC vc;
            PC pc;
            constraint_ctor(x, item, b0, warm, dtRatio, vc, pc);
            float sep[2] = {0.0f, 0.0f};
            constraint_init_velocity(vc, pc, sb, sep);
            VRow vr = pack_v(vc, item);
            if (x.ws_mode && row_start_modes(x, item, kx + idx, vc, pc, sep, sb, h, vr))
                x.s_pend[c0 + atomicAdd(&wd.sw_npend, 1)] = idx;
            vrow[idx] = vr;
            if (njI || x.record_events) x.s_vpos[item] = idx;
            if (!njI) {
                prow[idx] = pack_p(pc, body_island[(bfl[vc.bodyA] & kBfStatic) ? vc.bodyB : vc.bodyA]);
                pdone = true;
            }
        } else {
            vrow[idx].ids = make_int4(0, 0, 0, item);
            if (x.ws_mode == 1) x.s_slog[kx + idx] = -1;
        }
        if (!pdone) {
            const int pitem = sched_p[kx + idx];
            const int is = item_island(x, pitem, b0);
            if (pitem >= 0) {
                VC vc;
                PC pc;
                constraint_ctor(x, pitem, b0, warm, dtRatio, vc, pc);
                prow[idx] = pack_p(pc, is);
            } else {
                prow[idx].ids = make_int4(0, 0, pitem, is);
            }
        }
    }
    csync();
    if (x.ws_mode == 2) {
        // predicted starts, 16 pending rows per tensor-core pass, kInferWarps warps of the first block
        const int warp = tid >> 5;
        if (r0 && warp < kInferWarps) {
            const int npend = ld_volatile_i(&wd.sw_npend);
            __nv_bfloat16* X = reinterpret_cast<__nv_bfloat16*>(big_smem) + (size_t)warp * kInferStage;
            for (int p0 = 16 * warp; p0 < npend; p0 += 16 * kInferWarps)
                infer_pending16(x, x.s_pend + c0, p0, npend, vrow, X, X + 16 * kFeat, X + 16 * kFeat + 16 * kHid);
        }
        csync();
    }
    stampb(4);
    auto sweep = [&](const int* lvl, int maxL, auto&& f) {             // levels in order over the block
        for (int L = 1; L <= maxL; ++L) {
            const int e = lvl[L + 1];
            for (int idx = lvl[L] + tid; idx < e; idx += nt) f(idx);
            __syncthreads();
        }
    };
    BigSweep bs_;
    bs_.b0 = b0;
    bs_.kx = kx;
    bs_.vrow = vrow;
    bs_.prow = prow;
    bs_.sb = sb;
    bs_.warm = warm;
    bs_.dtRatio = dtRatio;
    bs_.njI = njI;
    bs_.maxLv = maxLv;
    bs_.maxLp = maxLp;
    bs_.lvl_v = x.s_lvl_v + kx;
    bs_.lvl_p = lvl_p + kx;
    bs_.sched_p = sched_p;
    bs_.iflags = iflags;
    bs_.iminsep = iminsep;
    // warm start contacts, then joints' InitVelocityConstraints (b2island.d:133-146)
    if (njI == 0) {
        if (warm) cluster_levels(bs_.lvl_v, maxLv, gtid, gsize, clustered, r0, [&](int idx) { big_warm_row(x, bs_, idx); });
    } else {
        cluster_levels(bs_.lvl_p, maxLp, gtid, gsize, clustered, r0, [&](int idx) { big_warm_row(x, bs_, idx); });
    }
    stampb(5);
    // velocity iterations (b2island.d:153-161)
    for (int it = 0; it < x.vel_iters; ++it)
        cluster_levels(bs_.lvl_v, maxLv, gtid, gsize, clustered, r0, [&](int idx) { big_vel_row(x, bs_, idx, it); });
    stampb(6);
    if (x.measure && r0) {
        // one extra velocity sweep that changes nothing: velocities kept aside and put back,
        // impulses not written, joints left out
        for (int t = tid; t < nbI; t += nt) {
            const int i = isl_body[t];
            const float2 v = sb.v(i);
            x.s_vsave[3 * (size_t)(b0 + i)] = v.x;
            x.s_vsave[3 * (size_t)(b0 + i) + 1] = v.y;
            x.s_vsave[3 * (size_t)(b0 + i) + 2] = sb.w(i);
        }
        __syncthreads();
        float ssq = 0.0f, smax = 0.0f;
        int npts = 0;
        sweep(x.s_lvl_v + kx, maxLv, [&](int idx) {
            const VRow r = load_v(vrow + idx);
            if (r.ids.w < 0) return;
            VC vc = unpack_v(r);
            const VC before = vc;
            solve_velocity(vc, sb);
            for (int j = 0; j < vc.pointCount; ++j) {
                const float dn = vc.p[j].normalImpulse - before.p[j].normalImpulse;
                const float dt = vc.p[j].tangentImpulse - before.p[j].tangentImpulse;
                const float d2 = dn * dn + dt * dt;
                ssq += d2;
                smax = bmax(smax, sqrtf(d2));
                ++npts;
            }
        });
        auto fsum = [](float a, float b) { return a + b; };
        auto fmx = [](float a, float b) { return bmax(a, b); };
        auto isum = [](int a, int b) { return a + b; };
        ssq = block_reduce(ssq, fsum, shf);
        smax = block_reduce(smax, fmx, shf);
        npts = block_reduce(npts, isum, shi);
        if (tid == 0) { wd.q_sumsq = ssq; wd.q_max = smax; wd.q_points = npts; }
        __syncthreads();
        for (int t = tid; t < nbI; t += nt) {
            const int i = isl_body[t];
            const float* sv = x.s_vsave + 3 * (size_t)(b0 + i);
            sb.set_v(i, v2(sv[0], sv[1]), sv[2]);
        }
        __syncthreads();
    }
    if (x.measure) csync();
    for (int idx = gtid; idx < nItems; idx += gsize) {                   // StoreImpulses (b2contactsolver.d:774-787)
        const VRow r = load_v(vrow + idx);
        if (r.ids.w >= 0) store_impulses(x, r);
        if (x.ws_mode == 1) {                                            // a logged sample's targets
            const int slot = x.s_slog[kx + idx];
            if (slot >= 0) {
                float* tg = x.samples + (size_t)kSampleFloats * slot + kFeat;
                tg[0] = r.imp.x; tg[1] = r.imp.y; tg[2] = r.imp.z; tg[3] = r.imp.w;
            }
        }
    }
    // integrate positions (b2island.d:168-200)
    for (int t = gtid; t < nbI; t += gsize) {
        const int i = isl_body[t];
        float2 c = sb.c(i);
        float a = sb.a(i);
        float2 v = sb.v(i);
        float wv = sb.w(i);
        float2 translation = h * v;
        if (dot(translation, translation) > kMaxTranslationSquared) {
            float ratio = fdiv(kMaxTranslation, length(translation));
            v *= ratio;
        }
        float rotation = h * wv;
        if (rotation * rotation > kMaxRotationSquared) {
            float ratio = fdiv(kMaxRotation, babs(rotation));
            wv *= ratio;
        }
        c += h * v;
        a += h * wv;
        sb.set_c(i, c, a);
        sb.set_v(i, v, wv);
    }
    for (int is = gtid; is < nIsl; is += gsize) iflags[is] = 0;
    csync();                                                           // positions integrated
    stampb(7);
    // position iterations with per-island early exit (b2island.d:206-224)
    for (int it = 0; it < x.pos_iters; ++it) {
        for (int is = gtid; is < nIsl; is += gsize) {
            iminsep[is] = fkey(0.0f);
            iflags[is] &= ~4;
        }
        csync();
        cluster_levels(bs_.lvl_p, maxLp, gtid, gsize, clustered, r0, [&](int idx) { big_pos_row(x, bs_, idx); });
        bool go = false;
        if (r0) {                                                      // the islands' checks
        int psolved = 0;
        bool remaining = false;
        for (int is = tid; is < nIsl; is += nt) {
            const int f = iflags[is];
            if (f & 1) continue;
            psolved += x.s_isl_cstart[bx + is + 1] - x.s_isl_cstart[bx + is];
            const bool contactsOkay = funkey(iminsep[is]) >= -3.0f * kLinearSlop;
            const bool jointsOkay = (f & 4) == 0;
            if (contactsOkay && jointsOkay) iflags[is] = f | 1 | 2;
            else remaining = true;
        }
        auto isum = [](int a, int b) { return a + b; };
        psolved = block_reduce(psolved, isum, shi);
        if (tid == 0) wd.acc_psolve += (unsigned long long)psolved;
        go = __syncthreads_or(remaining) != 0;
        if (tid == 0) wd.sw_go = go ? 1 : 0;
        }                                                              // r0
        csync();
        if (!r0) go = ld_volatile_i(&wd.sw_go) != 0;
        if (!go) break;
    }
    csync();
    if (x.measure && r0) {
        float ms = 0.0f;
        for (int idx = tid; idx < nItems; idx += nt) {
            const PRow r = load_p(prow + idx);
            if (r.ids.z >= 0) ms = bmin(ms, position_min_separation(unpack_p(r), sb));
        }
        auto fmn = [](float a, float b) { return bmin(a, b); };
        ms = block_reduce(ms, fmn, shf);
        if (tid == 0) wd.q_minsep = ms;
    }
    if (x.record_events && r0) {
        // b2Island.Report (b2island.d:419-438): PostSolve per island contact in island order
        const int e0 = wd.ev_count;
        for (int t = tid; t < ncI; t += nt) {
            const int item = isl_contact[t];
            const VRow r = load_v(vrow + x.s_vpos[item]);
            float ni[2] = {r.imp.x, r.imp.z}, ti[2] = {r.imp.y, r.imp.w};
            put_event(x, wi, w, e0 + t, DBOX_EVENT_POSTSOLVE, x.ct[item], r.ids.z & 0xff, ni, ti);
        }
        __syncthreads();
        if (tid == 0) wd.ev_count = e0 + ncI;
    }
    stampb(8);
    // copy back + SynchronizeTransform (b2island.d:227-235)
    bool nonfinite = false;
    for (int t = gtid; t < nbI; t += gsize) {
        const int i = isl_body[t];
        dbox_body_state& B = x.bs[b0 + i];
        const float2 c = sb.c(i), v = sb.v(i);
        B.sweep[4] = c.x; B.sweep[5] = c.y; B.sweep[7] = sb.a(i);
        B.vel[0] = v.x; B.vel[1] = v.y; B.vel[2] = sb.w(i);
        b_sync_transform(B);
        nonfinite |= !(isfinite(c.x) && isfinite(c.y) && isfinite(B.sweep[7]) && isfinite(v.x) && isfinite(v.y) &&
                       isfinite(B.vel[2]));
    }
    if (nonfinite) set_error(x, w, DBOX_ERR_NAN);
    csync();
    // sleep (b2island.d:241-279)
    if (x.allow_sleep) {
        const float linTolSqr = kLinearSleepTolerance * kLinearSleepTolerance;
        const float angTolSqr = kAngularSleepTolerance * kAngularSleepTolerance;
        for (int is = gtid; is < nIsl; is += gsize) x.s_isl_sleep[b0 + is] = fkey(kMaxFloat);
        csync();
        for (int t = gtid; t < nbI; t += gsize) {
            const int i = isl_body[t];
            dbox_body_state& B = x.bs[b0 + i];
            const int is = body_island[i];
            if ((B.flags & kBodyAutoSleep) == 0 || B.vel[2] * B.vel[2] > angTolSqr || dot(b_v(B), b_v(B)) > linTolSqr) {
                B.sleep_time = 0.0f;
                atomicMin(&x.s_isl_sleep[b0 + is], fkey(0.0f));
            } else {
                B.sleep_time += h;
                atomicMin(&x.s_isl_sleep[b0 + is], fkey(B.sleep_time));
            }
        }
        csync();
        for (int is = gtid; is < nIsl; is += gsize) {
            const int f = iflags[is];
            if (funkey(x.s_isl_sleep[b0 + is]) >= kTimeToSleep && (f & 2)) iflags[is] = f | 8;
        }
        csync();
        for (int t = gtid; t < nbI; t += gsize) {
            const int i = isl_body[t];
            if (iflags[body_island[i]] & 8) b_set_awake(x.bs[b0 + i], false);
        }
        // a static body ends in the state its last island left it in
        for (int i = gtid; i < nb; i += gsize) {
            if ((bfl[i] & kBfStatic) && body_island[i] >= 0 && (iflags[body_island[i]] & 8))
                b_set_awake(x.bs[b0 + i], false);
        }
    }
    stampb(9);
    stampb(10);
    stampb(11);
}

// The solve phase and the TOI phase of one step, one warp per world: each world goes
// from its island solve straight to its TOI events, so a world that is slow in one phase
// overlaps with worlds that are slow in the other.  Worlds reach warps in one of two ways:
// the host's packing of worlds into blocks (solve_world / solve_smem per warp slot), or a
// queue: one resident wave of warps takes worlds costliest first, with the heavy worlds
// spread one per SM sub-partition so that two long dependent chains do not share an issue
// slot.  Each warp's shared memory holds its row staging and, when the world fits, the
// world's solver body rows.
constexpr int kQueueWaitLimit = 1 << 16;      // bounded wait of the exclusive queue mode (x 2 us)

DG int ld_acquire_int(const int* p) { return *reinterpret_cast<const volatile int*>(p); }

// kFused: the whole step, x.steps times over, for each world the warp takes (k_step_fused)
template <bool kFused>
DG void solve_warps(const Ctx& x) {
    extern __shared__ float smem_sb[];
    const int warp = threadIdx.x >> 5, lane = lane_id();
    const int slot = blockIdx.x * x.solve_wpb + warp;
    const bool queued = x.solve_queue != nullptr;
    float* stage_f;
    float* own = nullptr;
    if (queued) {
        stage_f = smem_sb + warp * (kWarpSmemFloats + 8 * x.solve_cap);
        own = stage_f + kWarpSmemFloats;
    } else {
        stage_f = smem_sb + warp * kWarpSmemFloats;
    }
    // the warp's row ring: its two barriers are initialised once, before the first world
    RowRing ring;
    ring.base = stage_f;
    ring.bar = reinterpret_cast<unsigned long long*>(stage_f + kStageFloats);
    ring.par = 0;
    ring.ok = true;
    ring.budget = x.wait_polls;
    if (lane == 0) {
        mbar_init(&ring.bar[0]);
        mbar_init(&ring.bar[1]);
        fence_mbar_init();
    }
    tsync();
    int sub = -1;                                      // this warp's SM sub-partition (queue mode)
    if (queued && lane == 0) {
        unsigned smid, warpid;
        asm volatile("mov.u32 %0, %%smid;" : "=r"(smid));
        asm volatile("mov.u32 %0, %%warpid;" : "=r"(warpid));
        if ((int)smid < x.solve_nsm) sub = 4 * (int)smid + (int)(warpid & 3u);
    }
    for (int round = 0;; ++round) {
        int w = -1, heavy = 0;
        if (!queued) {
            if (round > 0) break;
            w = x.solve_world[slot];
        } else {
            if (lane == 0) {
                int* q = x.solve_queue;
                const int H = x.solve_heavy, nl = x.W - H;
                if (H > 0 && sub >= 0 && ld_acquire_int(&q[0]) < H && atomicCAS(&q[2 + sub], 0, 1) == 0) {
                    const int i = atomicAdd(&q[0], 1);
                    if (i < H) { w = x.solve_order[i]; heavy = 1; }
                    else atomicExch(&q[2 + sub], 0);
                }
                if (w < 0) {
                    if (x.solve_exclusive && sub >= 0)
                        for (int k = 0; k < kQueueWaitLimit && ld_acquire_int(&q[2 + sub]) != 0 &&
                                        ld_acquire_int(&q[1]) < nl; ++k)
                            __nanosleep(2000);
                    const int i = atomicAdd(&q[1], 1);
                    if (i < nl) w = x.solve_order[H + i];
                }
            }
            w = __shfl_sync(0xffffffffu, w, 0);
            heavy = __shfl_sync(0xffffffffu, heavy, 0);
        }
        if (w < 0) break;
        float* sbp;
        bool in_smem;
        if (queued) {
            in_smem = x.wi[w].body_count <= x.solve_cap;
            sbp = in_smem ? own : x.s_sbody + 6 * (size_t)x.wi[w].body_start;
        } else {
            const int soff = x.solve_smem[slot];
            in_smem = soff >= 0;
            sbp = in_smem ? smem_sb + soff : x.s_sbody + 6 * (size_t)x.wi[w].body_start;
        }
        unsigned long long g0 = 0;
        if (x.prof) asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(g0));
        if constexpr (kFused) {                                          // no large worlds in this launch
            for (int st = 0; st < x.steps; ++st) {
                collide_world(x, w);
                solve_world(x, w, sbp, in_smem, stage_f, ring);
                tsync();
                toi_world(x, w, sbp);
                tsync();
            }
        } else {
            if (!(x.big_block && x.wi[w].pair_block)) solve_world(x, w, sbp, in_smem, stage_f, ring);   // else k_solve_big
            tsync();
            if (!x.wi[w].pair_block) toi_world(x, w, sbp);               // large worlds: k_toi_big
            tsync();
        }
        if (heavy && lane == 0) atomicExch(&x.solve_queue[2 + sub], 0);
        if (x.prof && lane == 0 && !(x.big_block && x.wi[w].pair_block)) {
            unsigned long long g1;
            asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(g1));
            x.prof[kProfSlots * (size_t)w + 25] = g0;
            x.prof[kProfSlots * (size_t)w + 26] = g1;
            x.prof[kProfSlots * (size_t)w + 27] = slot;
            unsigned smid, warpid;
            asm volatile("mov.u32 %0, %%smid;" : "=r"(smid));
            asm volatile("mov.u32 %0, %%warpid;" : "=r"(warpid));
            x.prof[kProfSlots * (size_t)w + 28] = smid;
            x.prof[kProfSlots * (size_t)w + 29] = warpid;
            if (!x.wi[w].pair_block) x.prof[kProfSlots * (size_t)w + 15] = in_smem ? 1 : 0;
        }
    }
}

__global__ void __launch_bounds__(kSolveWarps * 32, 3) k_solve_toi(const __grid_constant__ Ctx x) { solve_warps<false>(x); }

// One launch for x.steps whole steps of every world (a handle without large worlds): each warp
// takes its worlds through their steps one after the other (b2World.Step of separate worlds
// shares nothing), so a world never waits at a step boundary for the others, and the deep
// worlds start their solve right after their own Collide
__global__ void __launch_bounds__(kSolveWarps * 32, 3) k_step_fused(const __grid_constant__ Ctx x) { solve_warps<true>(x); }

}  // namespace dg

// ------------------------------------------------------------ launch entry points (called from api.cpp)
// Launch one step.  ev, when not NULL, holds 4 events recorded at the phase
// boundaries: [0] before Collide, [1] before Solve, [2] and [3] after Solve + SolveTOI (one kernel).
// part 1 of a step: FindNewContacts for new fixtures, then Collide (3 launches)
// a large-world kernel on a cluster of x->big_cluster blocks per world (its passes spread over
// them), or on one block
template <class K>
static void launch_big(K kernel, const dg::Ctx* x, unsigned threads, size_t smem, cudaStream_t stream) {
    const int c = x->big_cluster > 1 ? x->big_cluster : 1;
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((unsigned)(x->n_big * c));
    cfg.blockDim = dim3(threads);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = stream;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = (unsigned)c;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.attrs = attr;
    cfg.numAttrs = c > 1 ? 1 : 0;
    cudaLaunchKernelEx(&cfg, kernel, *x);
}
static void launch_solve_big(const dg::Ctx* x, cudaStream_t stream) {
    launch_big(dg::k_solve_big, x, dg::kBigThreads, x->ws_mode == 2 ? dg::kBigSmemInfer : 0, stream);
}

extern "C" int dbox_launch_collide(const dg::Ctx* x, cudaStream_t stream) {
    const int threads = 128;                       // four worlds per block, one warp each
    int team_blocks = (x->W * dg::kWarp + threads - 1) / threads;
    int flat_blocks = (x->total_contacts + 255) / 256;
    if (flat_blocks < 1) flat_blocks = 1;
    if (flat_blocks > 152 * 16) flat_blocks = 152 * 16;
    dg::k_step_begin<<<team_blocks, threads, 0, stream>>>(*x);
    if (x->n_big > 0) dg::k_begin_big<<<x->n_big, dg::kPairThreads, 0, stream>>>(*x);
    dg::k_collide<<<flat_blocks, 256, 0, stream>>>(*x);
    dg::k_collide_finish<<<team_blocks, threads, 0, stream>>>(*x);
    if (x->n_big > 0) launch_big(dg::k_collide_finish_big, x, dg::kPairThreads, 0, stream);
    return (int)cudaGetLastError();
}


// part 2 of a step: Solve and SolveTOI (1 launch, 4 or 5 with a large world); *launches = all of the step's
// (part 1 is 3 launches, 5 with a large world)
extern "C" int dbox_launch_solve(const dg::Ctx* x, cudaStream_t stream, int* launches) {
    if (x->solve_blocks < 1) return (int)cudaErrorInvalidValue;
    if (x->solve_queue) cudaMemsetAsync(x->solve_queue, 0, sizeof(int) * (2 + 4 * (size_t)x->solve_nsm), stream);
    if (x->big_block) launch_solve_big(x, stream);  // large worlds' Solve
    dg::k_solve_toi<<<x->solve_blocks, x->solve_wpb * dg::kWarp, x->solve_smem_floats * sizeof(float), stream>>>(*x);
    if (x->n_big > 0) {                             // large worlds: pairs and AddPair on their clusters, then TOI
        launch_big(dg::k_pairs_block, x, dg::kPairThreads, 0, stream);
        launch_big(dg::k_finish_big_block, x, dg::kPairThreads, 0, stream);
        dg::k_toi_big<<<x->n_big, dg::kToiThreads, 0, stream>>>(*x);
    }
    if (launches) *launches = x->n_big > 0 ? 9 + x->big_block : 4;
    return (int)cudaGetLastError();
}

extern "C" int dbox_launch_step_ev(const dg::Ctx* x, cudaStream_t stream, int* launches, cudaEvent_t* ev) {
    const int threads = 128;                       // four worlds per block, one warp each
    int team_blocks = (x->W * dg::kWarp + threads - 1) / threads;
    if (x->solve_blocks < 1) return (int)cudaErrorInvalidValue;
    int flat_blocks = (x->total_contacts + 255) / 256;
    if (flat_blocks < 1) flat_blocks = 1;
    if (flat_blocks > 152 * 16) flat_blocks = 152 * 16;
    if (ev) cudaEventRecordWithFlags(ev[0], stream, cudaEventRecordExternal);
    dg::k_step_begin<<<team_blocks, threads, 0, stream>>>(*x);
    if (x->n_big > 0) dg::k_begin_big<<<x->n_big, dg::kPairThreads, 0, stream>>>(*x);
    dg::k_collide<<<flat_blocks, 256, 0, stream>>>(*x);
    dg::k_collide_finish<<<team_blocks, threads, 0, stream>>>(*x);
    if (x->n_big > 0) launch_big(dg::k_collide_finish_big, x, dg::kPairThreads, 0, stream);
    if (ev) cudaEventRecordWithFlags(ev[1], stream, cudaEventRecordExternal);
    if (x->solve_queue) cudaMemsetAsync(x->solve_queue, 0, sizeof(int) * (2 + 4 * (size_t)x->solve_nsm), stream);
    if (x->big_block) launch_solve_big(x, stream);  // large worlds' Solve
    dg::k_solve_toi<<<x->solve_blocks, x->solve_wpb * dg::kWarp, x->solve_smem_floats * sizeof(float), stream>>>(*x);
    if (x->n_big > 0) {                             // large worlds: pairs and AddPair on their clusters, then TOI
        launch_big(dg::k_pairs_block, x, dg::kPairThreads, 0, stream);
        launch_big(dg::k_finish_big_block, x, dg::kPairThreads, 0, stream);
        dg::k_toi_big<<<x->n_big, dg::kToiThreads, 0, stream>>>(*x);
    }
    if (ev) cudaEventRecordWithFlags(ev[2], stream, cudaEventRecordExternal);
    if (ev) cudaEventRecordWithFlags(ev[3], stream, cudaEventRecordExternal);
    if (launches) *launches = x->n_big > 0 ? 9 + x->big_block : 4;
    return (int)cudaGetLastError();
}

extern "C" const void* dbox_solve_kernel() { return reinterpret_cast<const void*>(&dg::k_solve_toi); }
extern "C" const void* dbox_step_fused_kernel() { return reinterpret_cast<const void*>(&dg::k_step_fused); }

// x->steps whole steps of every world in one launch (k_step_fused; a handle without large
// worlds); *launches = 1
extern "C" int dbox_launch_steps_fused(const dg::Ctx* x, cudaStream_t stream, int* launches) {
    if (x->solve_blocks < 1 || x->n_big > 0 || x->steps < 1) return (int)cudaErrorInvalidValue;
    if (x->solve_queue) cudaMemsetAsync(x->solve_queue, 0, sizeof(int) * (2 + 4 * (size_t)x->solve_nsm), stream);
    dg::k_step_fused<<<x->solve_blocks, x->solve_wpb * dg::kWarp, x->solve_smem_floats * sizeof(float), stream>>>(*x);
    if (launches) *launches = 1;
    return (int)cudaGetLastError();
}
// the largest cluster (8, 4, 2 or 1 blocks) that k_solve_big can run on this device
extern "C" int dbox_big_solve_init(int* cluster) {
    int rc = (int)cudaFuncSetAttribute(dg::k_solve_big, cudaFuncAttributeMaxDynamicSharedMemorySize, dg::kBigSmemInfer);
    *cluster = 1;
    if (rc) return rc;
    for (int c = 8; c > 1; c /= 2) {
        cudaLaunchConfig_t cfg = {};
        cfg.gridDim = dim3((unsigned)c);
        cfg.blockDim = dim3(dg::kBigThreads);
        cfg.dynamicSmemBytes = dg::kBigSmemInfer;
        cudaLaunchAttribute attr[1];
        attr[0].id = cudaLaunchAttributeClusterDimension;
        attr[0].val.clusterDim.x = (unsigned)c;
        attr[0].val.clusterDim.y = 1;
        attr[0].val.clusterDim.z = 1;
        cfg.attrs = attr;
        cfg.numAttrs = 1;
        int n = 0;
        if (cudaOccupancyMaxActiveClusters(&n, dg::k_solve_big, &cfg) == cudaSuccess && n >= 1) { *cluster = c; break; }
        cudaGetLastError();
    }
    return 0;
}

extern "C" int dbox_launch_step(const dg::Ctx* x, cudaStream_t stream, int* launches) {
    return dbox_launch_step_ev(x, stream, launches, nullptr);
}

// ------------------------------------------------------------ bulk host I/O
namespace dg {
// b2Body.GetPosition / GetAngle for every body: (x, y, angle) triples
__global__ void k_gather_transforms(int n, const dbox_body_state* bs, float* out) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        out[3 * i + 0] = bs[i].xf[0];
        out[3 * i + 1] = bs[i].xf[1];
        out[3 * i + 2] = bs[i].sweep[7];
    }
}
// b2Body.ApplyForceToCenter + ApplyTorque with wake = false (b2body.d:360-420): accumulate on awake dynamic bodies
__global__ void k_apply_forces(int n, dbox_body_state* bs, const float* f) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        dbox_body_state& b = bs[i];
        if (b.type != kDynamicBody || (b.flags & kBodyAwake) == 0) continue;
        b.force[0] += f[3 * i + 0];
        b.force[1] += f[3 * i + 1];
        b.force[2] += f[3 * i + 2];
    }
}
}  // namespace dg

extern "C" int dbox_launch_gather_transforms(int n, const dbox_body_state* bs, float* out, cudaStream_t s) {
    if (n <= 0) return 0;
    int blocks = (n + 255) / 256;
    if (blocks > 152 * 8) blocks = 152 * 8;
    dg::k_gather_transforms<<<blocks, 256, 0, s>>>(n, bs, out);
    return (int)cudaGetLastError();
}
extern "C" int dbox_launch_apply_forces(int n, dbox_body_state* bs, const float* f, cudaStream_t s) {
    if (n <= 0) return 0;
    int blocks = (n + 255) / 256;
    if (blocks > 152 * 8) blocks = 152 * 8;
    dg::k_apply_forces<<<blocks, 256, 0, s>>>(n, bs, f);
    return (int)cudaGetLastError();
}

// ------------------------------------------------------------ standalone narrowphase
namespace dg {
// One thread per shape pair: the manifold of b2CollidePolygons / b2CollidePolygonAndCircle /
// b2CollideCircles (fixture a must be the polygon of a mixed pair).
__global__ void k_collide_pairs(int n, const DFixture* fa, const float4* xa, const DFixture* fb, const float4* xb,
                                dbox_contact_state* out) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        Xf A, B;
        float4 a = xa[i], b = xb[i];
        A.p = v2(a.x, a.y); A.q.s = a.z; A.q.c = a.w;
        B.p = v2(b.x, b.y); B.q.s = b.z; B.q.c = b.w;
        Manifold m;
        manifold_load(out[i], m);
        evaluate_manifold(m, fa[i], A, fb[i], B);
        manifold_store(m, out[i]);
    }
}
}  // namespace dg

extern "C" int dbox_launch_collide_pairs(int n, const dg::DFixture* fa, const float4* xa, const dg::DFixture* fb,
                                         const float4* xb, dbox_contact_state* out, cudaStream_t stream) {
    int blocks = (n + 127) / 128;
    if (blocks < 1) blocks = 1;
    dg::k_collide_pairs<<<blocks, 128, 0, stream>>>(n, fa, xa, fb, xb, out);
    return (int)cudaGetLastError();
}
