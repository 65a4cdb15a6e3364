// Device float32 geometry for the b2World.Step kernels: vector algebra,
// shape AABBs, narrowphase manifolds, GJK distance and time of impact.
//
// Every function keeps the reference's operation order (dbox src/dbox/...,
// cited per function) and the library is compiled with --fmad=false,
// -prec-div=true, -prec-sqrt=true, so each operation rounds once exactly as
// the reference's IEEE binary32 arithmetic does.  b2Min/b2Max/b2Abs use the
// reference's comparison forms, not fminf/fmaxf (their NaN rules differ).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>
#include <float.h>

#include "dbox_trig.h"
#include "../../include/dbox_gpu.h"

namespace dg {

#define DG __device__ __forceinline__

// ------------------------------------------------------------ constants (common/b2settings.d:61-149)
constexpr float kMaxFloat = FLT_MAX;
constexpr float kEpsilon = FLT_EPSILON;
constexpr float kPi = 3.14159265359f;
constexpr float kAabbExtension = 0.1f;
constexpr float kAabbMultiplier = 2.0f;
constexpr float kLinearSlop = 0.005f;
constexpr float kAngularSlop = (2.0f / 180.0f * kPi);
constexpr float kPolygonRadius = (2.0f * kLinearSlop);
constexpr int kMaxSubSteps = 8;
constexpr int kMaxTOIContacts = 32;
constexpr float kVelocityThreshold = 1.0f;
constexpr float kMaxLinearCorrection = 0.2f;
constexpr float kMaxAngularCorrection = (8.0f / 180.0f * kPi);
constexpr float kMaxTranslation = 2.0f;
constexpr float kMaxTranslationSquared = (kMaxTranslation * kMaxTranslation);
constexpr float kMaxRotation = (0.5f * kPi);
constexpr float kMaxRotationSquared = (kMaxRotation * kMaxRotation);
constexpr float kBaumgarte = 0.2f;
constexpr float kToiBaumgarte = 0.75f;
constexpr float kTimeToSleep = 0.5f;
constexpr float kLinearSleepTolerance = 0.01f;
constexpr float kAngularSleepTolerance = (2.0f / 180.0f * kPi);

enum { kStaticBody = 0, kKinematicBody = 1, kDynamicBody = 2 };
enum { kShapeCircle = 0, kShapeEdge = 1, kShapePolygon = 2 };
enum { kBodyIsland = 0x1, kBodyAwake = 0x2, kBodyAutoSleep = 0x4, kBodyBullet = 0x8, kBodyFixedRotation = 0x10,
       kBodyActive = 0x20 };
enum { kContactIsland = 0x1, kContactTouching = 0x2, kContactEnabled = 0x4, kContactFilter = 0x8,
       kContactBulletHit = 0x10, kContactToi = 0x20,
       // learned warm start only (never set in the plain method): manifold point 0 / 1 had no
       // feature-id match in the last update, so its impulse started from zero
       kContactNew0 = 0x40, kContactNew1 = 0x80,
       // set by the host's PreSolve window when the callback disabled the contact; the sub-step
       // updates of SolveTOI keep it disabled, the next Collide clears it
       kContactUserOff = 0x100 };
enum { kManifoldCircles = 0, kManifoldFaceA = 1, kManifoldFaceB = 2 };

// ------------------------------------------------------------ vector algebra (common/b2math.d)
DG float2 v2(float x, float y) { return make_float2(x, y); }
DG float2 operator+(float2 a, float2 b) { return v2(a.x + b.x, a.y + b.y); }
DG float2 operator-(float2 a, float2 b) { return v2(a.x - b.x, a.y - b.y); }
DG float2 operator-(float2 a) { return v2(-a.x, -a.y); }
DG float2 operator*(float s, float2 v) { return v2(s * v.x, s * v.y); }
DG void operator+=(float2& a, float2 b) { a.x += b.x; a.y += b.y; }
DG void operator-=(float2& a, float2 b) { a.x -= b.x; a.y -= b.y; }
DG void operator*=(float2& a, float s) { a.x *= s; a.y *= s; }
DG float dot(float2 a, float2 b) { return a.x * b.x + a.y * b.y; }
DG float cross(float2 a, float2 b) { return a.x * b.y - a.y * b.x; }
DG float2 cross(float2 a, float s) { return v2(s * a.y, -s * a.x); }
DG float2 cross(float s, float2 a) { return v2(-s * a.y, s * a.x); }
DG float bmin(float a, float b) { return a < b ? a : b; }
DG float bmax(float a, float b) { return a > b ? a : b; }
DG float babs(float a) { return a > 0.0f ? a : -a; }
DG float bclamp(float a, float lo, float hi) { return bmax(lo, bmin(a, hi)); }
DG float2 vmin(float2 a, float2 b) { return v2(bmin(a.x, b.x), bmin(a.y, b.y)); }
DG float2 vmax(float2 a, float2 b) { return v2(bmax(a.x, b.x), bmax(a.y, b.y)); }
DG float fsqrt(float x) { return __fsqrt_rn(x); }
DG float fdiv(float a, float b) { return __fdiv_rn(a, b); }
DG float length(float2 v) { return fsqrt(v.x * v.x + v.y * v.y); }
DG float length_sq(float2 v) { return v.x * v.x + v.y * v.y; }
DG float dist_sq(float2 a, float2 b) { float2 c = a - b; return dot(c, c); }
DG float dist(float2 a, float2 b) { return length(a - b); }
DG float normalize(float2& v) {                                        // b2math.d:160-175
    float len = length(v);
    if (len < kEpsilon) return 0.0f;
    float inv = fdiv(1.0f, len);
    v.x *= inv;
    v.y *= inv;
    return len;
}

struct Rot { float s, c; };
struct Xf { float2 p; Rot q; };

DG Rot rot(float angle) { Rot r; dbox_sincosf(angle, &r.s, &r.c); return r; }
DG float2 mul(Rot q, float2 v) { return v2(q.c * v.x - q.s * v.y, q.s * v.x + q.c * v.y); }
DG float2 mulT(Rot q, float2 v) { return v2(q.c * v.x + q.s * v.y, -q.s * v.x + q.c * v.y); }
DG Rot mulT(Rot q, Rot r) { Rot o; o.s = q.c * r.s - q.s * r.c; o.c = q.c * r.c + q.s * r.s; return o; }
DG float2 mul(const Xf& T, float2 v) {                                 // b2math.d:734-740
    float x = (T.q.c * v.x - T.q.s * v.y) + T.p.x;
    float y = (T.q.s * v.x + T.q.c * v.y) + T.p.y;
    return v2(x, y);
}
DG float2 mulT(const Xf& T, float2 v) {                                // b2math.d:743-751
    float px = v.x - T.p.x;
    float py = v.y - T.p.y;
    return v2(T.q.c * px + T.q.s * py, -T.q.s * px + T.q.c * py);
}
DG Xf mulT(const Xf& A, const Xf& B) { Xf C; C.q = mulT(A.q, B.q); C.p = mulT(A.q, B.p - A.p); return C; }

// b2Sweep (b2math.d:554-593): localCenter, c0, c, a0, a, alpha0
struct Sweep { float2 lc, c0, c; float a0, a, alpha0; };
DG void sweep_xf(const Sweep& s, Xf* xf, float beta) {
    xf->p = (1.0f - beta) * s.c0 + beta * s.c;
    float angle = (1.0f - beta) * s.a0 + beta * s.a;
    xf->q = rot(angle);
    xf->p -= mul(xf->q, s.lc);
}
DG void sweep_advance(Sweep& s, float alpha) {
    float beta = fdiv(alpha - s.alpha0, 1.0f - s.alpha0);
    s.c0 += beta * (s.c - s.c0);
    s.a0 += beta * (s.a - s.a0);
    s.alpha0 = alpha;
}
DG void sweep_normalize(Sweep& s) {
    float twoPi = 2.0f * kPi;
    float d = twoPi * floorf(fdiv(s.a0, twoPi));
    s.a0 -= d;
    s.a -= d;
}

// ------------------------------------------------------------ shapes
// Device fixture record: shape + material + filter.  For a circle, v[0] is m_p; for an edge,
// v[0], v[1] are m_vertex1, m_vertex2 (count 2) and v[2], v[3] the ghost vertices m_vertex0,
// m_vertex3 when edge_flags has bit 0 (hasVertex0) / bit 1 (hasVertex3).
struct DFixture {
    int body;          // global body index
    int type;          // kShapeCircle / kShapeEdge / kShapePolygon
    int count;         // polygon vertex count (1 for a circle, 2 for an edge)
    float radius;
    float friction, restitution, density;
    int sensor;
    uint32_t filter;   // categoryBits | maskBits << 16
    int group;         // groupIndex
    float2 centroid;   // polygon centroid (b2polygonshape.d:561-565)
    float2 v[8];
    float2 n[8];
    int edge_flags;
    int fclass;        // filter class 0..63 of a table contact filter (dbox_world_set_contact_filter)
};

struct AABB { float2 lo, hi; };

DG AABB fixture_aabb(const DFixture& f, const Xf& xf) {
    AABB a;
    if (f.type == kShapeCircle) {                                      // b2circleshape.d:110-117
        float2 p = xf.p + mul(xf.q, f.v[0]);
        a.lo = v2(p.x - f.radius, p.y - f.radius);
        a.hi = v2(p.x + f.radius, p.y + f.radius);
        return a;
    }
    float2 lower = mul(xf, f.v[0]);                                    // b2polygonshape.d:356-373
    float2 upper = lower;
    for (int i = 1; i < f.count; ++i) {
        float2 v = mul(xf, f.v[i]);
        lower = vmin(lower, v);
        upper = vmax(upper, v);
    }
    float2 r = v2(f.radius, f.radius);
    a.lo = lower - r;
    a.hi = upper + r;
    return a;
}

DG bool aabb_overlap(const AABB& a, const AABB& b) {                   // b2collision.d:470-483
    float2 d1 = b.lo - a.hi;
    float2 d2 = a.lo - b.hi;
    if (d1.x > 0.0f || d1.y > 0.0f) return false;
    if (d2.x > 0.0f || d2.y > 0.0f) return false;
    return true;
}
DG bool aabb_contains(const AABB& outer, const AABB& a) {              // b2collision.d:329-337
    bool r = true;
    r = r && outer.lo.x <= a.lo.x;
    r = r && outer.lo.y <= a.lo.y;
    r = r && a.hi.x <= outer.hi.x;
    r = r && a.hi.y <= outer.hi.y;
    return r;
}

// ------------------------------------------------------------ manifold (b2collision.d:38-114)
// Field names follow dbox_contact_state; local points are stored as float pairs.
struct Manifold {
    int pointCount;
    int type;
    float2 localNormal;
    float2 localPoint;
    float2 lp[2];
    float ni[2], ti[2];
    uint32_t id[2];
};

DG void manifold_load(const dbox_contact_state& c, Manifold& m) {
    m.pointCount = c.point_count;
    m.type = c.type;
    m.localNormal = v2(c.local_normal[0], c.local_normal[1]);
    m.localPoint = v2(c.local_point[0], c.local_point[1]);
    for (int k = 0; k < 2; ++k) {
        m.lp[k] = v2(c.points[k].local_point[0], c.points[k].local_point[1]);
        m.ni[k] = c.points[k].normal_impulse;
        m.ti[k] = c.points[k].tangent_impulse;
        m.id[k] = c.points[k].id;
    }
}
DG void manifold_store(const Manifold& m, dbox_contact_state& c) {
    c.point_count = m.pointCount;
    c.type = m.type;
    c.local_normal[0] = m.localNormal.x; c.local_normal[1] = m.localNormal.y;
    c.local_point[0] = m.localPoint.x; c.local_point[1] = m.localPoint.y;
    for (int k = 0; k < 2; ++k) {
        c.points[k].local_point[0] = m.lp[k].x; c.points[k].local_point[1] = m.lp[k].y;
        c.points[k].normal_impulse = m.ni[k];
        c.points[k].tangent_impulse = m.ti[k];
        c.points[k].id = m.id[k];
    }
}

DG uint32_t make_id(uint32_t ia, uint32_t ib, uint32_t ta, uint32_t tb) {
    return (ia & 0xffu) | ((ib & 0xffu) << 8) | ((ta & 0xffu) << 16) | ((tb & 0xffu) << 24);
}
enum { kFeatureVertex = 0, kFeatureFace = 1 };

struct ClipVertex { float2 v; uint32_t id; };

DG int clip_segment(ClipVertex vOut[2], const ClipVertex vIn[2], float2 normal, float offset, int vertexIndexA) {
    int numOut = 0;                                                     // b2collision.d:413-446
    float distance0 = dot(normal, vIn[0].v) - offset;
    float distance1 = dot(normal, vIn[1].v) - offset;
    if (distance0 <= 0.0f) vOut[numOut++] = vIn[0];
    if (distance1 <= 0.0f) vOut[numOut++] = vIn[1];
    if (distance0 * distance1 < 0.0f) {
        float interp = fdiv(distance0, distance0 - distance1);
        vOut[numOut].v = vIn[0].v + interp * (vIn[1].v - vIn[0].v);
        uint32_t ib = (vIn[0].id >> 8) & 0xffu;
        vOut[numOut].id = make_id((uint32_t)vertexIndexA, ib, kFeatureVertex, kFeatureFace);
        ++numOut;
    }
    return numOut;
}

DG float find_max_separation(int* edgeIndex, const DFixture& p1, const Xf& xf1, const DFixture& p2, const Xf& xf2) {
    Xf xf = mulT(xf2, xf1);                                            // b2collidepolygon.d:29-71
    int bestIndex = 0;
    float maxSeparation = -kMaxFloat;
    for (int i = 0; i < p1.count; ++i) {
        float2 n = mul(xf.q, p1.n[i]);
        float2 v1 = mul(xf, p1.v[i]);
        float si = kMaxFloat;
        for (int j = 0; j < p2.count; ++j) {
            float sij = dot(n, p2.v[j] - v1);
            if (sij < si) si = sij;
        }
        if (si > maxSeparation) { maxSeparation = si; bestIndex = i; }
    }
    *edgeIndex = bestIndex;
    return maxSeparation;
}

DG void find_incident_edge(ClipVertex c[2], const DFixture& p1, const Xf& xf1, int edge1, const DFixture& p2,
                           const Xf& xf2) {                            // b2collidepolygon.d:73-118
    float2 normal1 = mulT(xf2.q, mul(xf1.q, p1.n[edge1]));
    int index = 0;
    float minDot = kMaxFloat;
    for (int i = 0; i < p2.count; ++i) {
        float d = dot(normal1, p2.n[i]);
        if (d < minDot) { minDot = d; index = i; }
    }
    int i1 = index;
    int i2 = i1 + 1 < p2.count ? i1 + 1 : 0;
    c[0].v = mul(xf2, p2.v[i1]);
    c[0].id = make_id((uint32_t)edge1, (uint32_t)i1, kFeatureFace, kFeatureVertex);
    c[1].v = mul(xf2, p2.v[i2]);
    c[1].id = make_id((uint32_t)edge1, (uint32_t)i2, kFeatureFace, kFeatureVertex);
}

DG void collide_polygons(Manifold& m, const DFixture& polyA, const Xf& xfA, const DFixture& polyB, const Xf& xfB) {
    m.pointCount = 0;                                                   // b2collidepolygon.d:127-254
    float totalRadius = polyA.radius + polyB.radius;
    int edgeA = 0;
    float separationA = find_max_separation(&edgeA, polyA, xfA, polyB, xfB);
    if (separationA > totalRadius) return;
    int edgeB = 0;
    float separationB = find_max_separation(&edgeB, polyB, xfB, polyA, xfA);
    if (separationB > totalRadius) return;
    const DFixture* poly1;
    const DFixture* poly2;
    Xf xf1, xf2;
    int edge1;
    int flip;
    const float k_tol = 0.1f * kLinearSlop;
    if (separationB > separationA + k_tol) {
        poly1 = &polyB; poly2 = &polyA; xf1 = xfB; xf2 = xfA; edge1 = edgeB;
        m.type = kManifoldFaceB;
        flip = 1;
    } else {
        poly1 = &polyA; poly2 = &polyB; xf1 = xfA; xf2 = xfB; edge1 = edgeA;
        m.type = kManifoldFaceA;
        flip = 0;
    }
    ClipVertex incidentEdge[2];
    find_incident_edge(incidentEdge, *poly1, xf1, edge1, *poly2, xf2);
    int count1 = poly1->count;
    int iv1 = edge1;
    int iv2 = edge1 + 1 < count1 ? edge1 + 1 : 0;
    float2 v11 = poly1->v[iv1];
    float2 v12 = poly1->v[iv2];
    float2 localTangent = v12 - v11;
    normalize(localTangent);
    float2 localNormal = cross(localTangent, 1.0f);
    float2 planePoint = 0.5f * (v11 + v12);
    float2 tangent = mul(xf1.q, localTangent);
    float2 normal = cross(tangent, 1.0f);
    v11 = mul(xf1, v11);
    v12 = mul(xf1, v12);
    float frontOffset = dot(normal, v11);
    float sideOffset1 = -dot(tangent, v11) + totalRadius;
    float sideOffset2 = dot(tangent, v12) + totalRadius;
    ClipVertex clipPoints1[2];
    ClipVertex clipPoints2[2];
    clipPoints1[0].v = v2(0.0f, 0.0f); clipPoints1[0].id = 0;
    clipPoints1[1] = clipPoints1[0];
    clipPoints2[0] = clipPoints1[0];
    clipPoints2[1] = clipPoints1[0];
    int np = clip_segment(clipPoints1, incidentEdge, -tangent, sideOffset1, iv1);
    if (np < 2) return;
    np = clip_segment(clipPoints2, clipPoints1, tangent, sideOffset2, iv2);
    if (np < 2) return;
    m.localNormal = localNormal;
    m.localPoint = planePoint;
    int pointCount = 0;
    for (int i = 0; i < 2; ++i) {
        float separation = dot(normal, clipPoints2[i].v) - frontOffset;
        if (separation <= totalRadius) {
            m.lp[pointCount] = mulT(xf2, clipPoints2[i].v);
            uint32_t id = clipPoints2[i].id;
            if (flip) {
                uint32_t ia = id & 0xffu, ib = (id >> 8) & 0xffu, ta = (id >> 16) & 0xffu, tb = (id >> 24) & 0xffu;
                id = make_id(ib, ia, tb, ta);
            }
            m.id[pointCount] = id;
            ++pointCount;
        }
    }
    m.pointCount = pointCount;
}

DG void collide_circles(Manifold& m, const DFixture& a, const Xf& xfA, const DFixture& b, const Xf& xfB) {
    m.pointCount = 0;                                                   // b2collidecircle.d:29-56
    float2 pA = mul(xfA, a.v[0]);
    float2 pB = mul(xfB, b.v[0]);
    float2 d = pB - pA;
    float distSqr = dot(d, d);
    float rA = a.radius, rB = b.radius;
    float radius = rA + rB;
    if (distSqr > radius * radius) return;
    m.type = kManifoldCircles;
    m.localPoint = a.v[0];
    m.localNormal = v2(0.0f, 0.0f);
    m.pointCount = 1;
    m.lp[0] = b.v[0];
    m.id[0] = 0;
}

DG void collide_polygon_circle(Manifold& m, const DFixture& polygonA, const Xf& xfA, const DFixture& circleB,
                               const Xf& xfB) {                        // b2collidecircle.d:59-164
    m.pointCount = 0;
    float2 c = mul(xfB, circleB.v[0]);
    float2 cLocal = mulT(xfA, c);
    int normalIndex = 0;
    float separation = -kMaxFloat;
    float radius = polygonA.radius + circleB.radius;
    int vertexCount = polygonA.count;
    for (int i = 0; i < vertexCount; ++i) {
        float s = dot(polygonA.n[i], cLocal - polygonA.v[i]);
        if (s > radius) return;
        if (s > separation) { separation = s; normalIndex = i; }
    }
    int vertIndex1 = normalIndex;
    int vertIndex2 = vertIndex1 + 1 < vertexCount ? vertIndex1 + 1 : 0;
    float2 v1 = polygonA.v[vertIndex1];
    float2 v2_ = polygonA.v[vertIndex2];
    if (separation < kEpsilon) {
        m.pointCount = 1;
        m.type = kManifoldFaceA;
        m.localNormal = polygonA.n[normalIndex];
        m.localPoint = 0.5f * (v1 + v2_);
        m.lp[0] = circleB.v[0];
        m.id[0] = 0;
        return;
    }
    float u1 = dot(cLocal - v1, v2_ - v1);
    float u2 = dot(cLocal - v2_, v1 - v2_);
    if (u1 <= 0.0f) {
        if (dist_sq(cLocal, v1) > radius * radius) return;
        m.pointCount = 1;
        m.type = kManifoldFaceA;
        m.localNormal = cLocal - v1;
        normalize(m.localNormal);
        m.localPoint = v1;
        m.lp[0] = circleB.v[0];
        m.id[0] = 0;
    } else if (u2 <= 0.0f) {
        if (dist_sq(cLocal, v2_) > radius * radius) return;
        m.pointCount = 1;
        m.type = kManifoldFaceA;
        m.localNormal = cLocal - v2_;
        normalize(m.localNormal);
        m.localPoint = v2_;
        m.lp[0] = circleB.v[0];
        m.id[0] = 0;
    } else {
        float2 faceCenter = 0.5f * (v1 + v2_);
        float separation2 = dot(cLocal - faceCenter, polygonA.n[vertIndex1]);
        if (separation2 > radius) return;
        m.pointCount = 1;
        m.type = kManifoldFaceA;
        m.localNormal = polygonA.n[vertIndex1];
        m.localPoint = faceCenter;
        m.lp[0] = circleB.v[0];
        m.id[0] = 0;
    }
}

// b2CollideEdgeAndCircle (collision/b2collideedge.d:31-155): the circle against the edge's
// regions A and B (vertices, unless an adjacent edge owns the region) and AB (the face)
static __device__ __noinline__ void collide_edge_circle(Manifold& m, const DFixture& edgeA, const Xf& xfA,
                                                 const DFixture& circleB, const Xf& xfB) {
    m.pointCount = 0;
    float2 Q = mulT(xfA, mul(xfB, circleB.v[0]));                     // circle in the edge's frame
    float2 A = edgeA.v[0], B = edgeA.v[1];
    float2 e = B - A;
    float u = dot(e, B - Q);                                            // barycentric coordinates
    float v = dot(e, Q - A);
    float radius = edgeA.radius + circleB.radius;
    if (v <= 0.0f) {                                                    // region A
        float2 d = Q - A;
        if (dot(d, d) > radius * radius) return;
        if (edgeA.edge_flags & 1) {
            float2 A1 = edgeA.v[2], B1 = A;
            float2 e1 = B1 - A1;
            if (dot(e1, B1 - Q) > 0.0f) return;                         // region AB of the previous edge
        }
        m.pointCount = 1;
        m.type = kManifoldCircles;
        m.localNormal = v2(0.0f, 0.0f);
        m.localPoint = A;
        m.lp[0] = circleB.v[0];
        m.id[0] = make_id(0u, 0u, kFeatureVertex, kFeatureVertex);
        return;
    }
    if (u <= 0.0f) {                                                    // region B
        float2 d = Q - B;
        if (dot(d, d) > radius * radius) return;
        if (edgeA.edge_flags & 2) {
            float2 B2 = edgeA.v[3], A2 = B;
            float2 e2 = B2 - A2;
            if (dot(e2, Q - A2) > 0.0f) return;                         // region AB of the next edge
        }
        m.pointCount = 1;
        m.type = kManifoldCircles;
        m.localNormal = v2(0.0f, 0.0f);
        m.localPoint = B;
        m.lp[0] = circleB.v[0];
        m.id[0] = make_id(1u, 0u, kFeatureVertex, kFeatureVertex);
        return;
    }
    float den = dot(e, e);                                              // region AB
    float2 P = fdiv(1.0f, den) * (u * A + v * B);
    float2 d = Q - P;
    if (dot(d, d) > radius * radius) return;
    float2 n = v2(-e.y, e.x);
    if (dot(n, Q - A) < 0.0f) n = v2(-n.x, -n.y);
    normalize(n);
    m.pointCount = 1;
    m.type = kManifoldFaceA;
    m.localNormal = n;
    m.localPoint = A;
    m.lp[0] = circleB.v[0];
    m.id[0] = make_id(0u, 0u, kFeatureFace, kFeatureVertex);
}

// b2EPCollider (collision/b2collideedge.d:157-717): an edge against a polygon, the edge's
// ghost vertices limiting the admissible normals
static __device__ __noinline__ void collide_edge_polygon(Manifold& m, const DFixture& edgeA, const Xf& xfA,
                                                  const DFixture& polygonB, const Xf& xfB) {
    enum { kUnknown = 0, kEdgeA = 1, kEdgeB = 2 };
    Xf xf = mulT(xfA, xfB);
    float2 centroidB = mul(xf, polygonB.centroid);
    float2 v0 = edgeA.v[2], v1 = edgeA.v[0], v2_ = edgeA.v[1], v3 = edgeA.v[3];
    const bool hasVertex0 = (edgeA.edge_flags & 1) != 0, hasVertex3 = (edgeA.edge_flags & 2) != 0;
    float2 edge1 = v2_ - v1;
    normalize(edge1);
    float2 normal0 = v2(0.0f, 0.0f), normal1 = v2(edge1.y, -edge1.x), normal2 = v2(0.0f, 0.0f);
    float offset1 = dot(normal1, centroidB - v1);
    float offset0 = 0.0f, offset2 = 0.0f;
    bool convex1 = false, convex2 = false;
    if (hasVertex0) {                                                   // a preceding edge
        float2 edge0 = v1 - v0;
        normalize(edge0);
        normal0 = v2(edge0.y, -edge0.x);
        convex1 = cross(edge0, edge1) >= 0.0f;
        offset0 = dot(normal0, centroidB - v0);
    }
    if (hasVertex3) {                                                   // a following edge
        float2 edge2 = v3 - v2_;
        normalize(edge2);
        normal2 = v2(edge2.y, -edge2.x);
        convex2 = cross(edge1, edge2) > 0.0f;
        offset2 = dot(normal2, centroidB - v2_);
    }
    // front or back collision; the collision normal and its limits
    bool front;
    float2 normal, lowerLimit, upperLimit;
    auto set = [&](bool f, float2 nf, float2 lf, float2 uf, float2 nb, float2 lb, float2 ub) {
        front = f;
        if (front) { normal = nf; lowerLimit = lf; upperLimit = uf; }
        else { normal = nb; lowerLimit = lb; upperLimit = ub; }
    };
    if (hasVertex0 && hasVertex3) {
        if (convex1 && convex2)
            set(offset0 >= 0.0f || offset1 >= 0.0f || offset2 >= 0.0f, normal1, normal0, normal2, -normal1, -normal1, -normal1);
        else if (convex1)
            set(offset0 >= 0.0f || (offset1 >= 0.0f && offset2 >= 0.0f), normal1, normal0, normal1, -normal1, -normal2, -normal1);
        else if (convex2)
            set(offset2 >= 0.0f || (offset0 >= 0.0f && offset1 >= 0.0f), normal1, normal1, normal2, -normal1, -normal1, -normal0);
        else
            set(offset0 >= 0.0f && offset1 >= 0.0f && offset2 >= 0.0f, normal1, normal1, normal1, -normal1, -normal2, -normal0);
    } else if (hasVertex0) {
        if (convex1) set(offset0 >= 0.0f || offset1 >= 0.0f, normal1, normal0, -normal1, -normal1, normal1, -normal1);
        else set(offset0 >= 0.0f && offset1 >= 0.0f, normal1, normal1, -normal1, -normal1, normal1, -normal0);
    } else if (hasVertex3) {
        if (convex2) set(offset1 >= 0.0f || offset2 >= 0.0f, normal1, -normal1, normal2, -normal1, -normal1, normal1);
        else set(offset1 >= 0.0f && offset2 >= 0.0f, normal1, -normal1, normal1, -normal1, -normal2, normal1);
    } else {
        set(offset1 >= 0.0f, normal1, -normal1, -normal1, -normal1, normal1, normal1);
    }
    float2 pv[8], pn[8];                                                // polygon B in frame A
    const int pcount = polygonB.count;
    for (int i = 0; i < pcount; ++i) {
        pv[i] = mul(xf, polygonB.v[i]);
        pn[i] = mul(xf.q, polygonB.n[i]);
    }
    const float radius = 2.0f * (2.0f * kLinearSlop);                   // 2 * b2_polygonRadius
    m.pointCount = 0;
    // edge separation (b2collideedge.d:636-653)
    int edgeType = kEdgeA, edgeIndex = front ? 0 : 1;
    float edgeSeparation = kMaxFloat;
    for (int i = 0; i < pcount; ++i) {
        float s = dot(normal, pv[i] - v1);
        if (s < edgeSeparation) edgeSeparation = s;
    }
    if (edgeSeparation > radius) return;
    // polygon separation (b2collideedge.d:655-700)
    int polyType = kUnknown, polyIndex = -1;
    float polySeparation = -kMaxFloat;
    {
        float2 perp = v2(-normal.y, normal.x);
        for (int i = 0; i < pcount; ++i) {
            float2 n = -pn[i];
            float s1 = dot(n, pv[i] - v1);
            float s2 = dot(n, pv[i] - v2_);
            float s = bmin(s1, s2);
            if (s > radius) { polyType = kEdgeB; polyIndex = i; polySeparation = s; break; }   // no collision
            if (dot(n, perp) >= 0.0f) {                                 // adjacency
                if (dot(n - upperLimit, normal) < -kAngularSlop) continue;
            } else {
                if (dot(n - lowerLimit, normal) < -kAngularSlop) continue;
            }
            if (s > polySeparation) { polyType = kEdgeB; polyIndex = i; polySeparation = s; }
        }
    }
    if (polyType != kUnknown && polySeparation > radius) return;
    const float k_relativeTol = 0.98f, k_absoluteTol = 0.001f;         // hysteresis
    int primaryType, primaryIndex;
    if (polyType == kUnknown) { primaryType = edgeType; primaryIndex = edgeIndex; }
    else if (polySeparation > k_relativeTol * edgeSeparation + k_absoluteTol) { primaryType = polyType; primaryIndex = polyIndex; }
    else { primaryType = edgeType; primaryIndex = edgeIndex; }
    ClipVertex ie[2];
    int rf_i1, rf_i2;
    float2 rf_v1, rf_v2, rf_normal;
    if (primaryType == kEdgeA) {
        m.type = kManifoldFaceA;
        int bestIndex = 0;                                              // the most anti-parallel polygon normal
        float bestValue = dot(normal, pn[0]);
        for (int i = 1; i < pcount; ++i) {
            float value = dot(normal, pn[i]);
            if (value < bestValue) { bestValue = value; bestIndex = i; }
        }
        int i1 = bestIndex;
        int i2 = i1 + 1 < pcount ? i1 + 1 : 0;
        ie[0].v = pv[i1];
        ie[0].id = make_id(0u, (uint32_t)i1, kFeatureFace, kFeatureVertex);
        ie[1].v = pv[i2];
        ie[1].id = make_id(0u, (uint32_t)i2, kFeatureFace, kFeatureVertex);
        if (front) { rf_i1 = 0; rf_i2 = 1; rf_v1 = v1; rf_v2 = v2_; rf_normal = normal1; }
        else { rf_i1 = 1; rf_i2 = 0; rf_v1 = v2_; rf_v2 = v1; rf_normal = -normal1; }
    } else {
        m.type = kManifoldFaceB;
        ie[0].v = v1;
        ie[0].id = make_id(0u, (uint32_t)primaryIndex, kFeatureVertex, kFeatureFace);
        ie[1].v = v2_;
        ie[1].id = make_id(0u, (uint32_t)primaryIndex, kFeatureVertex, kFeatureFace);
        rf_i1 = primaryIndex;
        rf_i2 = rf_i1 + 1 < pcount ? rf_i1 + 1 : 0;
        rf_v1 = pv[rf_i1];
        rf_v2 = pv[rf_i2];
        rf_normal = pn[rf_i1];
    }
    float2 sideNormal1 = v2(rf_normal.y, -rf_normal.x);
    float2 sideNormal2 = -sideNormal1;
    float sideOffset1 = dot(sideNormal1, rf_v1);
    float sideOffset2 = dot(sideNormal2, rf_v2);
    ClipVertex clipPoints1[2], clipPoints2[2];                          // clip against the side edges
    int np = clip_segment(clipPoints1, ie, sideNormal1, sideOffset1, rf_i1);
    if (np < 2) return;
    np = clip_segment(clipPoints2, clipPoints1, sideNormal2, sideOffset2, rf_i2);
    if (np < 2) return;
    if (primaryType == kEdgeA) {
        m.localNormal = rf_normal;
        m.localPoint = rf_v1;
    } else {
        m.localNormal = polygonB.n[rf_i1];
        m.localPoint = polygonB.v[rf_i1];
    }
    int pointCount = 0;
    for (int i = 0; i < 2; ++i) {
        float separation = dot(rf_normal, clipPoints2[i].v - rf_v1);
        if (separation <= radius) {
            if (primaryType == kEdgeA) {
                m.lp[pointCount] = mulT(xf, clipPoints2[i].v);
                m.id[pointCount] = clipPoints2[i].id;
            } else {
                uint32_t id = clipPoints2[i].id;
                uint32_t ia = id & 0xffu, ib = (id >> 8) & 0xffu, ta = (id >> 16) & 0xffu, tb = (id >> 24) & 0xffu;
                m.lp[pointCount] = clipPoints2[i].v;
                m.id[pointCount] = make_id(ib, ia, tb, ta);
            }
            ++pointCount;
        }
    }
    m.pointCount = pointCount;
}

// Shape-pair dispatch of b2PolygonContact / b2PolygonAndCircleContact / b2CircleContact /
// b2EdgeAndCircleContact / b2EdgeAndPolygonContact (contacts/b2polygoncontact.d:56-61 and
// siblings).  Fixture A is the "primary" type.
DG void evaluate_manifold(Manifold& m, const DFixture& fa, const Xf& xfA, const DFixture& fb, const Xf& xfB) {
    if (fa.type == kShapePolygon && fb.type == kShapePolygon) collide_polygons(m, fa, xfA, fb, xfB);
    else if (fa.type == kShapePolygon) collide_polygon_circle(m, fa, xfA, fb, xfB);
    else if (fa.type == kShapeEdge && fb.type == kShapeCircle) collide_edge_circle(m, fa, xfA, fb, xfB);
    else if (fa.type == kShapeEdge) collide_edge_polygon(m, fa, xfA, fb, xfB);
    else collide_circles(m, fa, xfA, fb, xfB);
}

// ------------------------------------------------------------ GJK distance (collision/b2distance.d)
struct Proxy { const float2* v; int count; float radius; };
DG Proxy make_proxy(const DFixture& f) { Proxy p; p.v = f.v; p.count = f.type == kShapeCircle ? 1 : f.count; p.radius = f.radius; return p; }
DG int support(const Proxy& p, float2 d) {
    int best = 0;
    float bestValue = dot(p.v[0], d);
    for (int i = 1; i < p.count; ++i) {
        float value = dot(p.v[i], d);
        if (value > bestValue) { best = i; bestValue = value; }
    }
    return best;
}

struct SimplexCache { float metric; int count; uint8_t ia[3], ib[3]; };
struct SimplexVertex { float2 wA, wB, w; float a; int ia, ib; };

struct Simplex {
    SimplexVertex v[3];
    int count;
    DG float metric() const {
        if (count == 1) return 0.0f;
        if (count == 2) return dist(v[0].w, v[1].w);
        if (count == 3) return cross(v[1].w - v[0].w, v[2].w - v[0].w);
        return 0.0f;
    }
    DG void read_cache(const SimplexCache& cache, const Proxy& pA, const Xf& xA, const Proxy& pB, const Xf& xB) {
        count = cache.count;                                            // b2distance.d:577-626
        for (int i = 0; i < count; ++i) {
            SimplexVertex& s = v[i];
            s.ia = cache.ia[i];
            s.ib = cache.ib[i];
            s.wA = mul(xA, pA.v[s.ia]);
            s.wB = mul(xB, pB.v[s.ib]);
            s.w = s.wB - s.wA;
            s.a = 0.0f;
        }
        if (count > 1) {
            float metric1 = cache.metric;
            float metric2 = metric();
            if (metric2 < 0.5f * metric1 || 2.0f * metric1 < metric2 || metric2 < kEpsilon) count = 0;
        }
        if (count == 0) {
            SimplexVertex& s = v[0];
            s.ia = 0;
            s.ib = 0;
            s.wA = mul(xA, pA.v[0]);
            s.wB = mul(xB, pB.v[0]);
            s.w = s.wB - s.wA;
            s.a = 1.0f;
            count = 1;
        }
    }
    DG void write_cache(SimplexCache& cache) const {
        cache.metric = metric();
        cache.count = count;
        for (int i = 0; i < count; ++i) { cache.ia[i] = (uint8_t)v[i].ia; cache.ib[i] = (uint8_t)v[i].ib; }
    }
    DG float2 search_direction() const {
        if (count == 1) return -v[0].w;
        float2 e12 = v[1].w - v[0].w;
        float sgn = cross(e12, -v[0].w);
        if (sgn > 0.0f) return cross(1.0f, e12);
        return cross(e12, 1.0f);
    }
    DG void witness(float2* pA, float2* pB) const {
        if (count == 1) { *pA = v[0].wA; *pB = v[0].wB; }
        else if (count == 2) {
            *pA = v[0].a * v[0].wA + v[1].a * v[1].wA;
            *pB = v[0].a * v[0].wB + v[1].a * v[1].wB;
        } else if (count == 3) {
            *pA = (v[0].a * v[0].wA + v[1].a * v[1].wA) + v[2].a * v[2].wA;
            *pB = *pA;
        }
    }
    DG void solve2() {                                                  // b2distance.d:388-423
        float2 w1 = v[0].w, w2 = v[1].w;
        float2 e12 = w2 - w1;
        float d12_2 = -dot(w1, e12);
        if (d12_2 <= 0.0f) { v[0].a = 1.0f; count = 1; return; }
        float d12_1 = dot(w2, e12);
        if (d12_1 <= 0.0f) { v[1].a = 1.0f; count = 1; v[0] = v[1]; return; }
        float inv = fdiv(1.0f, d12_1 + d12_2);
        v[0].a = d12_1 * inv;
        v[1].a = d12_2 * inv;
        count = 2;
    }
    DG void solve3() {                                                  // b2distance.d:430-575
        float2 w1 = v[0].w, w2 = v[1].w, w3 = v[2].w;
        float2 e12 = w2 - w1;
        float w1e12 = dot(w1, e12), w2e12 = dot(w2, e12);
        float d12_1 = w2e12, d12_2 = -w1e12;
        float2 e13 = w3 - w1;
        float w1e13 = dot(w1, e13), w3e13 = dot(w3, e13);
        float d13_1 = w3e13, d13_2 = -w1e13;
        float2 e23 = w3 - w2;
        float w2e23 = dot(w2, e23), w3e23 = dot(w3, e23);
        float d23_1 = w3e23, d23_2 = -w2e23;
        float n123 = cross(e12, e13);
        float d123_1 = n123 * cross(w2, w3);
        float d123_2 = n123 * cross(w3, w1);
        float d123_3 = n123 * cross(w1, w2);
        if (d12_2 <= 0.0f && d13_2 <= 0.0f) { v[0].a = 1.0f; count = 1; return; }
        if (d12_1 > 0.0f && d12_2 > 0.0f && d123_3 <= 0.0f) {
            float inv = fdiv(1.0f, d12_1 + d12_2);
            v[0].a = d12_1 * inv; v[1].a = d12_2 * inv; count = 2; return;
        }
        if (d13_1 > 0.0f && d13_2 > 0.0f && d123_2 <= 0.0f) {
            float inv = fdiv(1.0f, d13_1 + d13_2);
            v[0].a = d13_1 * inv; v[2].a = d13_2 * inv; count = 2; v[1] = v[2]; return;
        }
        if (d12_1 <= 0.0f && d23_2 <= 0.0f) { v[1].a = 1.0f; count = 1; v[0] = v[1]; return; }
        if (d13_1 <= 0.0f && d23_1 <= 0.0f) { v[2].a = 1.0f; count = 1; v[0] = v[2]; return; }
        if (d23_1 > 0.0f && d23_2 > 0.0f && d123_1 <= 0.0f) {
            float inv = fdiv(1.0f, d23_1 + d23_2);
            v[1].a = d23_1 * inv; v[2].a = d23_2 * inv; count = 2; v[0] = v[2]; return;
        }
        float inv = fdiv(1.0f, (d123_1 + d123_2) + d123_3);
        v[0].a = d123_1 * inv; v[1].a = d123_2 * inv; v[2].a = d123_3 * inv;
        count = 3;
    }
};

// b2Distance (b2distance.d:185-350); returns distance, witness points via out params.
// Out of line (like the separation-function members and time_of_impact below): each is
// large and called from several places, and inlined copies crowd the instruction cache of
// the fused solve kernel, whose warps run different phases side by side.
static __device__ __noinline__ float gjk_distance(SimplexCache& cache, const Proxy& pA, const Xf& xA, const Proxy& pB, const Xf& xB,
                      bool useRadii, float2* outA, float2* outB) {
    Simplex simplex;
    simplex.read_cache(cache, pA, xA, pB, xB);
    int saveA[3], saveB[3];
    int iter = 0;
    while (iter < 20) {
        int saveCount = simplex.count;
        for (int i = 0; i < saveCount; ++i) { saveA[i] = simplex.v[i].ia; saveB[i] = simplex.v[i].ib; }
        if (simplex.count == 2) simplex.solve2();
        else if (simplex.count == 3) simplex.solve3();
        if (simplex.count == 3) break;
        float2 d = simplex.search_direction();
        if (length_sq(d) < kEpsilon * kEpsilon) break;
        SimplexVertex& vx = simplex.v[simplex.count];
        vx.ia = support(pA, mulT(xA.q, -d));
        vx.wA = mul(xA, pA.v[vx.ia]);
        vx.ib = support(pB, mulT(xB.q, d));
        vx.wB = mul(xB, pB.v[vx.ib]);
        vx.w = vx.wB - vx.wA;
        ++iter;
        bool duplicate = false;
        for (int i = 0; i < saveCount; ++i) {
            if (vx.ia == saveA[i] && vx.ib == saveB[i]) { duplicate = true; break; }
        }
        if (duplicate) break;
        ++simplex.count;
    }
    float2 wa, wb;
    simplex.witness(&wa, &wb);
    float distance = dist(wa, wb);
    simplex.write_cache(cache);
    if (useRadii) {
        float rA = pA.radius, rB = pB.radius;
        if (distance > rA + rB && distance > kEpsilon) {
            distance -= rA + rB;
            float2 normal = wb - wa;
            normalize(normal);
            wa += rA * normal;
            wb -= rB * normal;
        } else {
            float2 p = 0.5f * (wa + wb);
            wa = p;
            wb = p;
            distance = 0.0f;
        }
    }
    if (outA) *outA = wa;
    if (outB) *outB = wb;
    return distance;
}

// b2TestOverlap(shapes) (b2collision.d:449-467)
DG bool shapes_overlap(const DFixture& a, const Xf& xA, const DFixture& b, const Xf& xB) {
    SimplexCache cache;
    cache.count = 0;
    cache.metric = 0.0f;
    float d = gjk_distance(cache, make_proxy(a), xA, make_proxy(b), xB, true, nullptr, nullptr);
    return d < 10.0f * kEpsilon;
}

// ------------------------------------------------------------ time of impact (collision/b2timeofimpact.d)
enum { kToiUnknown = 0, kToiFailed, kToiOverlapped, kToiTouching, kToiSeparated };
enum { kSepPoints = 0, kSepFaceA, kSepFaceB };

struct SepFn {
    Proxy pA, pB;
    Sweep sA, sB;
    int type;
    float2 localPoint, axis;
    __device__ __noinline__ void init(const SimplexCache& cache, const Proxy& a, const Sweep& sa, const Proxy& b, const Sweep& sb, float t1) {
        pA = a; pB = b;                                                 // b2timeofimpact.d:323-407
        int count = cache.count;
        sA = sa; sB = sb;
        Xf xfA, xfB;
        sweep_xf(sA, &xfA, t1);
        sweep_xf(sB, &xfB, t1);
        if (count == 1) {
            type = kSepPoints;
            float2 pointA = mul(xfA, pA.v[cache.ia[0]]);
            float2 pointB = mul(xfB, pB.v[cache.ib[0]]);
            axis = pointB - pointA;
            normalize(axis);
        } else if (cache.ia[0] == cache.ia[1]) {
            type = kSepFaceB;
            float2 b1 = pB.v[cache.ib[0]], b2 = pB.v[cache.ib[1]];
            axis = cross(b2 - b1, 1.0f);
            normalize(axis);
            float2 normal = mul(xfB.q, axis);
            localPoint = 0.5f * (b1 + b2);
            float2 pointB = mul(xfB, localPoint);
            float2 pointA = mul(xfA, pA.v[cache.ia[0]]);
            float s = dot(pointA - pointB, normal);
            if (s < 0.0f) axis = -axis;
        } else {
            type = kSepFaceA;
            float2 a1 = pA.v[cache.ia[0]], a2 = pA.v[cache.ia[1]];
            axis = cross(a2 - a1, 1.0f);
            normalize(axis);
            float2 normal = mul(xfA.q, axis);
            localPoint = 0.5f * (a1 + a2);
            float2 pointA = mul(xfA, localPoint);
            float2 pointB = mul(xfB, pB.v[cache.ib[0]]);
            float s = dot(pointB - pointA, normal);
            if (s < 0.0f) axis = -axis;
        }
    }
    __device__ __noinline__ float find_min(int* ia, int* ib, float t) const {                // b2timeofimpact.d:410-474
        Xf xfA, xfB;
        sweep_xf(sA, &xfA, t);
        sweep_xf(sB, &xfB, t);
        if (type == kSepPoints) {
            float2 axisA = mulT(xfA.q, axis);
            float2 axisB = mulT(xfB.q, -axis);
            *ia = support(pA, axisA);
            *ib = support(pB, axisB);
            float2 pointA = mul(xfA, pA.v[*ia]);
            float2 pointB = mul(xfB, pB.v[*ib]);
            return dot(pointB - pointA, axis);
        } else if (type == kSepFaceA) {
            float2 normal = mul(xfA.q, axis);
            float2 pointA = mul(xfA, localPoint);
            float2 axisB = mulT(xfB.q, -normal);
            *ia = -1;
            *ib = support(pB, axisB);
            float2 pointB = mul(xfB, pB.v[*ib]);
            return dot(pointB - pointA, normal);
        } else {
            float2 normal = mul(xfB.q, axis);
            float2 pointB = mul(xfB, localPoint);
            float2 axisA = mulT(xfA.q, -normal);
            *ib = -1;
            *ia = support(pA, axisA);
            float2 pointA = mul(xfA, pA.v[*ia]);
            return dot(pointA - pointB, normal);
        }
    }
    __device__ __noinline__ float evaluate(int ia, int ib, float t) const {                  // b2timeofimpact.d:477-519
        Xf xfA, xfB;
        sweep_xf(sA, &xfA, t);
        sweep_xf(sB, &xfB, t);
        if (type == kSepPoints) {
            float2 pointA = mul(xfA, pA.v[ia]);
            float2 pointB = mul(xfB, pB.v[ib]);
            return dot(pointB - pointA, axis);
        } else if (type == kSepFaceA) {
            float2 normal = mul(xfA.q, axis);
            float2 pointA = mul(xfA, localPoint);
            float2 pointB = mul(xfB, pB.v[ib]);
            return dot(pointB - pointA, normal);
        } else {
            float2 normal = mul(xfB.q, axis);
            float2 pointB = mul(xfB, localPoint);
            float2 pointA = mul(xfA, pA.v[ia]);
            return dot(pointA - pointB, normal);
        }
    }
};

// b2TimeOfImpact (b2timeofimpact.d:67-302) with tMax = 1.  Returns the state; *t receives output.t.
static __device__ __noinline__ int time_of_impact(const Proxy& pA, const Proxy& pB, Sweep sweepA, Sweep sweepB, float tMax, float* tOut) {
    int state = kToiUnknown;
    float tres = tMax;
    sweep_normalize(sweepA);
    sweep_normalize(sweepB);
    float totalRadius = pA.radius + pB.radius;
    float target = bmax(kLinearSlop, totalRadius - 3.0f * kLinearSlop);
    float tolerance = 0.25f * kLinearSlop;
    float t1 = 0.0f;
    int iter = 0;
    SimplexCache cache;
    cache.count = 0;
    cache.metric = 0.0f;
    for (;;) {
        Xf xfA, xfB;
        sweep_xf(sweepA, &xfA, t1);
        sweep_xf(sweepB, &xfB, t1);
        float distance = gjk_distance(cache, pA, xfA, pB, xfB, false, nullptr, nullptr);
        if (distance <= 0.0f) { state = kToiOverlapped; tres = 0.0f; break; }
        if (distance < target + tolerance) { state = kToiTouching; tres = t1; break; }
        SepFn fcn;
        fcn.init(cache, pA, sweepA, pB, sweepB, t1);
        bool done = false;
        float t2 = tMax;
        int pushBackIter = 0;
        for (;;) {
            int ia, ib;
            float s2 = fcn.find_min(&ia, &ib, t2);
            if (s2 > target + tolerance) { state = kToiSeparated; tres = tMax; done = true; break; }
            if (s2 > target - tolerance) { t1 = t2; break; }
            float s1 = fcn.evaluate(ia, ib, t1);
            if (s1 < target - tolerance) { state = kToiFailed; tres = t1; done = true; break; }
            if (s1 <= target + tolerance) { state = kToiTouching; tres = t1; done = true; break; }
            int rootIterCount = 0;
            float a1 = t1, a2 = t2;
            for (;;) {
                float t;
                if (rootIterCount & 1) t = a1 + fdiv((target - s1) * (a2 - a1), s2 - s1);
                else t = 0.5f * (a1 + a2);
                ++rootIterCount;
                float s = fcn.evaluate(ia, ib, t);
                if (babs(s - target) < tolerance) { t2 = t; break; }
                if (s > target) { a1 = t; s1 = s; } else { a2 = t; s2 = s; }
                if (rootIterCount == 50) break;
            }
            ++pushBackIter;
            if (pushBackIter == 8) break;
        }
        ++iter;
        if (done) break;
        if (iter == 20) { state = kToiFailed; tres = t1; break; }
    }
    *tOut = tres;
    return state;
}

}  // namespace dg
