// query.cu - batched world queries on the device: b2World.QueryAABB and b2World.RayCast
// (dynamics/b2world.d:563-587) over the broad-phase's fat AABBs.
//
// The reference walks its b2DynamicTree (collision/b2dynamictree.d:203-331) and hands each
// leaf to a callback.  The walk order depends on the tree's shape, which the GPU step does
// not keep (proxy ids and fat AABBs are kept bit-exact; the tree is not), so results are
// returned in fixture order and in the callback-independent forms the header states.
//
// Index (rebuilt per world when the step or an edit changed the proxies): the live proxies
// of a world sorted by the Morton code of their fat-AABB centre (12 bits per axis, a warp's
// stable 3-pass radix sort), then two levels of 32-wide unions: a bucket node covers 32
// consecutive proxies, a group node 32 buckets.  A query is one warp: each level is one
// coalesced 32-lane overlap test and a ballot, so a world of up to 32 x 32 x 32 proxies is
// three levels deep with no stack.  Hits are marked in a per-warp bitmap over the world's
// fixtures and emitted in fixture order by one pass over the bitmap, which also clears it.
#include <cuda_runtime.h>
#include <stdint.h>

#include "world.cuh"

namespace dg {
namespace {

constexpr int kQWarp = 32;
constexpr int kQWarpsPerBlock = 4;
constexpr unsigned kFull = 0xffffffffu;

DG int qlane() { return threadIdx.x & 31; }

struct QIndex {
    int W;
    const WorldInfo* wi;
    const DFixture* fx;
    const dbox_proxy_state* px;
    const dbox_body_state* bs;
    float4* box;        // fixture-indexed: fat AABBs of the live proxies in Morton order
    int* idx;           // fixture-indexed: world-local fixture index of each
    float4* bucket;     // per world from fix_start / 32 + world: unions of 32 proxies
    float4* group;      // per world from fix_start / 1024 + world: unions of 32 buckets
    int* live;          // per world: live proxies
    unsigned* key[2];   // fixture-indexed radix-sort ping-pong
    int* sidx[2];
    unsigned* bitmap;   // per query warp: bm_words words, all zero between queries
    int bm_words;
};

DG AABB f4_aabb(float4 b) { AABB a; a.lo = v2(b.x, b.y); a.hi = v2(b.z, b.w); return a; }

DG float4 union_reduce(float4 b) {
    for (int o = 16; o > 0; o >>= 1) {
        b.x = bmin(b.x, __shfl_xor_sync(kFull, b.x, o));
        b.y = bmin(b.y, __shfl_xor_sync(kFull, b.y, o));
        b.z = bmax(b.z, __shfl_xor_sync(kFull, b.z, o));
        b.w = bmax(b.w, __shfl_xor_sync(kFull, b.w, o));
    }
    return b;
}

DG unsigned spread12(unsigned v) {                 // 12 bits to the even bits of 24
    v &= 0xfffu;
    v = (v | (v << 8)) & 0x00ff00ffu;
    v = (v | (v << 4)) & 0x0f0f0f0fu;
    v = (v | (v << 2)) & 0x33333333u;
    v = (v | (v << 1)) & 0x55555555u;
    return v;
}

DG int quant12(float v, float o, float s) {
    float t = (v - o) * s;
    int q = (int)t;
    return q < 0 ? 0 : (q > 4095 ? 4095 : q);
}

// One warp per world: Morton sort of the live proxies, then the bucket and group unions.
__global__ void k_query_build(QIndex q) {
    __shared__ int hist_all[kQWarpsPerBlock][256];
    const int lane = qlane();
    const int w = blockIdx.x * kQWarpsPerBlock + (threadIdx.x >> 5);
    if (w >= q.W) return;
    int* hist = hist_all[threadIdx.x >> 5];
    const WorldInfo wi = q.wi[w];
    const int f0 = wi.fix_start, nf = wi.fix_count;
    float lo[2] = {3.4e38f, 3.4e38f}, hi[2] = {-3.4e38f, -3.4e38f};
    for (int i = lane; i < nf; i += kQWarp) {
        const dbox_proxy_state& p = q.px[f0 + i];
        if (p.proxy_id < 0) continue;
        for (int a = 0; a < 2; ++a) {
            float c = 0.5f * (p.fat_aabb[a] + p.fat_aabb[2 + a]);
            lo[a] = bmin(lo[a], c);
            hi[a] = bmax(hi[a], c);
        }
    }
    for (int o = 16; o > 0; o >>= 1)
        for (int a = 0; a < 2; ++a) {
            lo[a] = bmin(lo[a], __shfl_xor_sync(kFull, lo[a], o));
            hi[a] = bmax(hi[a], __shfl_xor_sync(kFull, hi[a], o));
        }
    const float span = bmax(bmax(hi[0] - lo[0], hi[1] - lo[1]), 1e-6f);
    const float scale = 4095.0f / span;
    unsigned* k0 = q.key[0] + f0;
    unsigned* k1 = q.key[1] + f0;
    int* i0 = q.sidx[0] + f0;
    int* i1 = q.sidx[1] + f0;
    int nv = 0;
    for (int base = 0; base < nf; base += kQWarp) {        // live proxies, in fixture order
        const int i = base + lane;
        const bool v = i < nf && q.px[f0 + i].proxy_id >= 0;
        const unsigned bal = __ballot_sync(kFull, v);
        if (v) {
            const dbox_proxy_state& p = q.px[f0 + i];
            const int r = nv + __popc(bal & ((1u << lane) - 1u));
            const float cx = 0.5f * (p.fat_aabb[0] + p.fat_aabb[2]), cy = 0.5f * (p.fat_aabb[1] + p.fat_aabb[3]);
            k0[r] = spread12((unsigned)quant12(cx, lo[0], scale)) | (spread12((unsigned)quant12(cy, lo[1], scale)) << 1);
            i0[r] = i;
        }
        nv += __popc(bal);
    }
    __syncwarp();
    for (int pass = 0; pass < 3; ++pass) {                 // stable LSD radix sort of 24-bit keys
        const int shift = 8 * pass;
        const unsigned* kin = pass & 1 ? k1 : k0;
        const int* iin = pass & 1 ? i1 : i0;
        unsigned* kout = pass & 1 ? k0 : k1;
        int* iout = pass & 1 ? i0 : i1;
        for (int b = lane; b < 256; b += kQWarp) hist[b] = 0;
        __syncwarp();
        for (int i = lane; i < nv; i += kQWarp) atomicAdd(&hist[(kin[i] >> shift) & 255u], 1);
        __syncwarp();
        int run = 0;
        for (int base = 0; base < 256; base += kQWarp) {
            const int v = hist[base + lane];
            int incl = v;
            for (int o = 1; o < 32; o <<= 1) {
                const int t = __shfl_up_sync(kFull, incl, o);
                if (lane >= o) incl += t;
            }
            hist[base + lane] = run + incl - v;
            run += __shfl_sync(kFull, incl, 31);
        }
        __syncwarp();
        for (int base = 0; base < nv; base += kQWarp) {
            const int i = base + lane;
            const unsigned k = i < nv ? kin[i] : 0u;
            const int d = i < nv ? (int)((k >> shift) & 255u) : 256 + lane;
            const unsigned peers = __match_any_sync(kFull, d);
            const unsigned below = peers & ((1u << lane) - 1u);
            if (i < nv) {
                const int pos = hist[d] + __popc(below);
                kout[pos] = k;
                iout[pos] = iin[i];
            }
            __syncwarp();
            if (i < nv && below == 0) hist[d] += __popc(peers);
            __syncwarp();
        }
    }
    // three passes: the sorted order is in the second buffer
    float4* box = q.box + f0;
    int* idx = q.idx + f0;
    for (int r = lane; r < nv; r += kQWarp) {
        const int i = i1[r];
        const dbox_proxy_state& p = q.px[f0 + i];
        box[r] = make_float4(p.fat_aabb[0], p.fat_aabb[1], p.fat_aabb[2], p.fat_aabb[3]);
        idx[r] = i;
    }
    __syncwarp();
    const float4 empty = make_float4(3.4e38f, 3.4e38f, -3.4e38f, -3.4e38f);
    const int nb = (nv + 31) >> 5, ng = (nb + 31) >> 5;
    float4* bucket = q.bucket + (f0 >> 5) + w;
    float4* group = q.group + (f0 >> 10) + w;
    for (int b = 0; b < nb; ++b) {
        const int r = b * 32 + lane;
        const float4 u = union_reduce(r < nv ? box[r] : empty);
        if (lane == 0) bucket[b] = u;
    }
    __syncwarp();
    for (int g = 0; g < ng; ++g) {
        const int b = g * 32 + lane;
        const float4 u = union_reduce(b < nb ? bucket[b] : empty);
        if (lane == 0) group[g] = u;
    }
    if (lane == 0) q.live[w] = nv;
}

// Walk the index of world w: fn(r) on every lane whose sorted proxy r lies in a bucket whose
// group and bucket unions pass node_test (each call runs with the whole warp converged; lanes
// without a proxy get r = -1).
template <class NodeTest, class Leaf>
DG void walk(const QIndex& q, int w, NodeTest node_test, Leaf fn) {
    const int lane = qlane();
    const int f0 = q.wi[w].fix_start;
    const int n = q.live[w], nb = (n + 31) >> 5, ng = (nb + 31) >> 5;
    const float4* bucket = q.bucket + (f0 >> 5) + w;
    const float4* group = q.group + (f0 >> 10) + w;
    for (int g0 = 0; g0 < ng; g0 += 32) {
        const int g = g0 + lane;
        unsigned mg = __ballot_sync(kFull, g < ng && node_test(group[g]));
        while (mg) {
            const int gg = g0 + __ffs(mg) - 1;
            mg &= mg - 1u;
            const int b = gg * 32 + lane;
            unsigned mb = __ballot_sync(kFull, b < nb && node_test(bucket[b]));
            while (mb) {
                const int bb = gg * 32 + __ffs(mb) - 1;
                mb &= mb - 1u;
                const int r = bb * 32 + lane;
                fn(r < n ? r : -1);
            }
        }
    }
}

// Ray casts of the three shape kinds (fraction and normal of b2RayCastOutput).
DG bool ray_circle(const DFixture& f, const Xf& xf, float2 p1, float2 p2, float maxf, float* frac, float2* nrm) {
    // b2circleshape.d:72-104
    const float2 position = xf.p + mul(xf.q, f.v[0]);
    const float2 s = p1 - position;
    const float b = dot(s, s) - f.radius * f.radius;
    const float2 r = p2 - p1;
    const float c = dot(s, r);
    const float rr = dot(r, r);
    const float sigma = c * c - rr * b;
    if (sigma < 0.0f || rr < kEpsilon) return false;
    float a = -(c + fsqrt(sigma));
    if (0.0f <= a && a <= maxf * rr) {
        a = fdiv(a, rr);
        *frac = a;
        float2 n = s + a * r;
        normalize(n);
        *nrm = n;
        return true;
    }
    return false;
}

DG bool ray_polygon(const DFixture& f, const Xf& xf, float2 rp1, float2 rp2, float maxf, float* frac, float2* nrm) {
    // b2polygonshape.d:283-351
    const float2 p1 = mulT(xf.q, rp1 - xf.p);
    const float2 p2 = mulT(xf.q, rp2 - xf.p);
    const float2 d = p2 - p1;
    float lower = 0.0f, upper = maxf;
    int index = -1;
    for (int i = 0; i < f.count; ++i) {
        const float numerator = dot(f.n[i], f.v[i] - p1);
        const float denominator = dot(f.n[i], d);
        if (denominator == 0.0f) {
            if (numerator < 0.0f) return false;
        } else if (denominator < 0.0f && numerator < lower * denominator) {
            lower = fdiv(numerator, denominator);
            index = i;
        } else if (denominator > 0.0f && numerator < upper * denominator) {
            upper = fdiv(numerator, denominator);
        }
        if (upper < lower) return false;
    }
    if (index >= 0) {
        *frac = lower;
        *nrm = mul(xf.q, f.n[index]);
        return true;
    }
    return false;
}

DG bool ray_edge(const DFixture& f, const Xf& xf, float2 rp1, float2 rp2, float maxf, float* frac, float2* nrm) {
    // b2edgeshape.d:96-157 (a chain child casts as its edge, b2chainshape.d:204-223)
    const float2 p1 = mulT(xf.q, rp1 - xf.p);
    const float2 p2 = mulT(xf.q, rp2 - xf.p);
    const float2 d = p2 - p1;
    const float2 va = f.v[0], vb = f.v[1];
    const float2 e = vb - va;
    float2 n = v2(e.y, -e.x);
    normalize(n);
    const float numerator = dot(n, va - p1);
    const float denominator = dot(n, d);
    if (denominator == 0.0f) return false;
    const float t = fdiv(numerator, denominator);
    if (t < 0.0f || maxf < t) return false;
    const float2 qp = p1 + t * d;
    const float2 r = vb - va;
    const float rr = dot(r, r);
    if (rr == 0.0f) return false;
    const float s = fdiv(dot(qp - va, r), rr);
    if (s < 0.0f || 1.0f < s) return false;
    *frac = t;
    const float2 wn = mul(xf.q, n);
    *nrm = numerator > 0.0f ? v2(-wn.x, -wn.y) : wn;
    return true;
}

DG bool ray_fixture(const QIndex& q, int f0, int fi, float2 p1, float2 p2, float* frac, float2* nrm) {
    const DFixture& f = q.fx[f0 + fi];
    const Xf xf = b_xf(q.bs[f.body]);
    if (f.type == kShapeCircle) return ray_circle(f, xf, p1, p2, 1.0f, frac, nrm);
    if (f.type == kShapeEdge) return ray_edge(f, xf, p1, p2, 1.0f, frac, nrm);
    return ray_polygon(f, xf, p1, p2, 1.0f, frac, nrm);
}

// Emit the marked fixtures of the warp's bitmap in fixture order (and clear it): fn(fi, pos)
// for each, pos counting from 0; returns the count.
template <class Emit>
DG int emit_bitmap(unsigned* bm, int words, Emit fn) {
    const int lane = qlane();
    int total = 0;
    for (int w0 = 0; w0 < words; w0 += 32) {
        const int wi = w0 + lane;
        unsigned bits = wi < words ? bm[wi] : 0u;
        if (bits) bm[wi] = 0u;
        const int c = __popc(bits);
        int incl = c;
        for (int o = 1; o < 32; o <<= 1) {
            const int t = __shfl_up_sync(kFull, incl, o);
            if (lane >= o) incl += t;
        }
        int pos = total + incl - c;
        while (bits) {
            const int b = __ffs(bits) - 1;
            bits &= bits - 1u;
            fn(wi * 32 + b, pos++);
        }
        total += __shfl_sync(kFull, incl, 31);
    }
    return total;
}

__global__ void k_query_aabb(QIndex q, int nq, const int* qworld, const dbox_aabb* boxes, int cap, int* counts,
                             int* out) {
    const int lane = qlane();
    const int gw = blockIdx.x * kQWarpsPerBlock + (threadIdx.x >> 5);
    const int nw = gridDim.x * kQWarpsPerBlock;
    unsigned* bm = q.bitmap + (size_t)gw * q.bm_words;
    for (int i = gw; i < nq; i += nw) {
        const int w = qworld[i];
        if (w < 0 || w >= q.W) {
            if (lane == 0) counts[i] = -1;
            continue;
        }
        const dbox_aabb qb = boxes[i];
        AABB a;
        a.lo = v2(qb.lower.x, qb.lower.y);
        a.hi = v2(qb.upper.x, qb.upper.y);
        const int f0 = q.wi[w].fix_start;
        const float4* box = q.box + f0;
        const int* idx = q.idx + f0;
        walk(q, w, [&](float4 nb) { return aabb_overlap(f4_aabb(nb), a); }, [&](int r) {
            if (r >= 0 && aabb_overlap(f4_aabb(box[r]), a)) {  // b2TestOverlap against the fat AABB
                const int fi = idx[r];
                atomicOr(&bm[fi >> 5], 1u << (fi & 31));
            }
        });
        __syncwarp();
        int* o = out + (size_t)i * cap;
        const int total = emit_bitmap(bm, (q.wi[w].fix_count + 31) >> 5, [&](int fi, int pos) {
            if (pos < cap) o[pos] = fi;
        });
        if (lane == 0) counts[i] = total;
        __syncwarp();
    }
}

struct Segment {
    float2 p1, p2, v, abs_v;
    AABB box;
};

// The segment data of b2DynamicTree.RayCast (b2dynamictree.d:246-276) with maxFraction 1.
DG Segment make_segment(float2 p1, float2 p2) {
    Segment s;
    s.p1 = p1;
    s.p2 = p2;
    float2 r = p2 - p1;
    normalize(r);
    s.v = cross(1.0f, r);
    s.abs_v = v2(babs(s.v.x), babs(s.v.y));
    const float2 t = p1 + 1.0f * (p2 - p1);
    s.box.lo = vmin(p1, t);
    s.box.hi = vmax(p1, t);
    return s;
}

// The tree's leaf test (b2dynamictree.d:283-297): overlap with the segment's box and the
// separating axis of the segment (Gino, p80).
DG bool segment_leaf(const Segment& s, float4 b) {
    const AABB a = f4_aabb(b);
    if (!aabb_overlap(a, s.box)) return false;
    const float2 c = 0.5f * (a.lo + a.hi);
    const float2 h = 0.5f * (a.hi - a.lo);
    const float separation = babs(dot(s.v, s.p1 - c)) - dot(s.abs_v, h);
    return !(separation > 0.0f);
}

DG void write_hit(dbox_ray_hit* o, int fi, const Segment& s, float frac, float2 nrm) {
    // b2WorldRayCastWrapper (b2world.d:1617-1619)
    const float2 point = (1.0f - frac) * s.p1 + frac * s.p2;
    dbox_ray_hit h;
    h.fixture = fi;
    h.fraction = frac;
    h.point.x = point.x;
    h.point.y = point.y;
    h.normal.x = nrm.x;
    h.normal.y = nrm.y;
    *o = h;
}

__global__ void k_raycast(QIndex q, int nq, const int* qworld, const dbox_vec2* p1s, const dbox_vec2* p2s, int mode,
                          int cap, int* counts, dbox_ray_hit* out) {
    const int lane = qlane();
    const int gw = blockIdx.x * kQWarpsPerBlock + (threadIdx.x >> 5);
    const int nw = gridDim.x * kQWarpsPerBlock;
    unsigned* bm = q.bitmap + (size_t)gw * q.bm_words;
    for (int i = gw; i < nq; i += nw) {
        const int w = qworld[i];
        const float2 p1 = v2(p1s[i].x, p1s[i].y), p2 = v2(p2s[i].x, p2s[i].y);
        const float2 r = p2 - p1;
        if (w < 0 || w >= q.W || !(dot(r, r) > 0.0f)) {
            if (lane == 0) counts[i] = -1;
            continue;
        }
        const Segment s = make_segment(p1, p2);
        const int f0 = q.wi[w].fix_start;
        const float4* box = q.box + f0;
        const int* idx = q.idx + f0;
        dbox_ray_hit* o = out + (size_t)i * cap;
        auto node_test = [&](float4 nb) { return aabb_overlap(f4_aabb(nb), s.box); };
        if (mode == DBOX_RAY_CLOSEST) {
            float best = 3.4e38f;
            int best_fi = 0x7fffffff;
            float2 best_n = v2(0.0f, 0.0f);
            walk(q, w, node_test, [&](int rr) {
                if (rr < 0 || !segment_leaf(s, box[rr])) return;
                const int fi = idx[rr];
                float frac;
                float2 nrm;
                if (ray_fixture(q, f0, fi, p1, p2, &frac, &nrm) && (frac < best || (frac == best && fi < best_fi))) {
                    best = frac;
                    best_fi = fi;
                    best_n = nrm;
                }
            });
            float wb = best;
            int wf = best_fi;
            for (int off = 16; off > 0; off >>= 1) {
                const float ob = __shfl_xor_sync(kFull, wb, off);
                const int of = __shfl_xor_sync(kFull, wf, off);
                if (ob < wb || (ob == wb && of < wf)) { wb = ob; wf = of; }
            }
            const bool found = wf != 0x7fffffff;
            if (found && best_fi == wf && best == wb) write_hit(o, wf, s, wb, best_n);   // the one lane holding it
            if (lane == 0) counts[i] = found ? 1 : 0;
        } else {
            walk(q, w, node_test, [&](int rr) {
                if (rr < 0 || !segment_leaf(s, box[rr])) return;
                const int fi = idx[rr];
                float frac;
                float2 nrm;
                if (ray_fixture(q, f0, fi, p1, p2, &frac, &nrm)) atomicOr(&bm[fi >> 5], 1u << (fi & 31));
            });
            __syncwarp();
            const int total = emit_bitmap(bm, (q.wi[w].fix_count + 31) >> 5, [&](int fi, int pos) {
                if (pos >= cap) return;
                float frac;
                float2 nrm;
                ray_fixture(q, f0, fi, p1, p2, &frac, &nrm);
                write_hit(o + pos, fi, s, frac, nrm);
            });
            if (lane == 0) counts[i] = total;
        }
        __syncwarp();
    }
}

}  // namespace
}  // namespace dg


static dg::QIndex qindex(const dbox_query_buffers* b) {
    dg::QIndex q;
    q.W = b->W;
    q.wi = b->wi;
    q.fx = b->fx;
    q.px = b->px;
    q.bs = b->bs;
    q.box = b->box;
    q.idx = b->idx;
    q.bucket = b->bucket;
    q.group = b->group;
    q.live = b->live;
    q.key[0] = b->key0;
    q.key[1] = b->key1;
    q.sidx[0] = b->sidx0;
    q.sidx[1] = b->sidx1;
    q.bitmap = b->bitmap;
    q.bm_words = b->bm_words;
    return q;
}

extern "C" int dbox_launch_query_build(const dbox_query_buffers* b, cudaStream_t s) {
    if (b->W <= 0) return 0;
    const int blocks = (b->W + dg::kQWarpsPerBlock - 1) / dg::kQWarpsPerBlock;
    dg::k_query_build<<<blocks, dg::kQWarpsPerBlock * 32, 0, s>>>(qindex(b));
    return (int)cudaGetLastError();
}

extern "C" int dbox_launch_query_aabb(const dbox_query_buffers* b, int n, const int* world, const dbox_aabb* boxes,
                                      int cap, int* counts, int* out, cudaStream_t s) {
    if (n <= 0) return 0;
    int blocks = (n + dg::kQWarpsPerBlock - 1) / dg::kQWarpsPerBlock;
    if (blocks > b->query_blocks) blocks = b->query_blocks;
    dg::k_query_aabb<<<blocks, dg::kQWarpsPerBlock * 32, 0, s>>>(qindex(b), n, world, boxes, cap, counts, out);
    return (int)cudaGetLastError();
}

extern "C" int dbox_launch_raycast(const dbox_query_buffers* b, int n, const int* world, const dbox_vec2* p1,
                                   const dbox_vec2* p2, int mode, int cap, int* counts, dbox_ray_hit* out,
                                   cudaStream_t s) {
    if (n <= 0) return 0;
    int blocks = (n + dg::kQWarpsPerBlock - 1) / dg::kQWarpsPerBlock;
    if (blocks > b->query_blocks) blocks = b->query_blocks;
    dg::k_raycast<<<blocks, dg::kQWarpsPerBlock * 32, 0, s>>>(qindex(b), n, world, p1, p2, mode, cap, counts, out);
    return (int)cudaGetLastError();
}

extern "C" int dbox_query_warps_per_block() { return dg::kQWarpsPerBlock; }
