// b2_oracle.cpp - TEST INFRASTRUCTURE ONLY (see b2_oracle.h).
//
// A CPU restatement of dbox's b2World.Step, written to follow the D sources
// operation by operation so that float32 results match the reference.  Every
// function cites the reference file:line it restates (paths within
// dbox/src/dbox/).  Build: -O2 -ffp-contract=off (no fused multiply-add, so
// each float operation rounds exactly once, as the reference's per-op IEEE
// binary32 arithmetic does).
//
// Structure mirrors the reference (linked lists, pointer graphs) on purpose:
// it is a checker, not a fast path.

#include "b2_oracle.h"
#include "../dbox_gb300/csrc/dbox_trig.h"

#include <math.h>
#include <float.h>
#include <string.h>
#include <stdlib.h>
#include <algorithm>
#include <cstdarg>
#include <string>
#include <vector>

namespace orc {

typedef float f32;

static int g_trig_mode = 0;  // 0: host libm sinf/cosf (reference), 1: dbox_sincosf

// ------------------------------------------------------------ settings
// common/b2settings.d:61-149
static const f32 kMaxFloat = FLT_MAX;
static const f32 kEpsilon = FLT_EPSILON;
static const f32 kPi = 3.14159265359f;
static const int kMaxManifoldPoints = 2;
static const int kMaxPolygonVertices = 8;
static const f32 kAabbExtension = 0.1f;
static const f32 kAabbMultiplier = 2.0f;
static const f32 kLinearSlop = 0.005f;
static const f32 kAngularSlop = (2.0f / 180.0f * kPi);
static const f32 kPolygonRadius = (2.0f * kLinearSlop);
static const int kMaxSubSteps = 8;
static const int kMaxTOIContacts = 32;
static const f32 kVelocityThreshold = 1.0f;
static const f32 kMaxLinearCorrection = 0.2f;
static const f32 kMaxAngularCorrection = (8.0f / 180.0f * kPi);
static const f32 kMaxTranslation = 2.0f;
static const f32 kMaxTranslationSquared = (kMaxTranslation * kMaxTranslation);
static const f32 kMaxRotation = (0.5f * kPi);
static const f32 kMaxRotationSquared = (kMaxRotation * kMaxRotation);
static const f32 kBaumgarte = 0.2f;
static const f32 kToiBaumgarte = 0.75f;
static const f32 kTimeToSleep = 0.5f;
static const f32 kLinearSleepTolerance = 0.01f;
static const f32 kAngularSleepTolerance = (2.0f / 180.0f * kPi);

// ------------------------------------------------------------ math
// common/b2math.d
struct Vec2 {
    f32 x = 0, y = 0;
    Vec2() {}
    Vec2(f32 x_, f32 y_) : x(x_), y(y_) {}
    void SetZero() { x = 0.0f; y = 0.0f; }
    void Set(f32 a, f32 b) { x = a; y = b; }
    Vec2 operator-() const { return Vec2(-x, -y); }
    void operator+=(Vec2 v) { x += v.x; y += v.y; }
    void operator-=(Vec2 v) { x -= v.x; y -= v.y; }
    void operator*=(f32 s) { x *= s; y *= s; }
    f32 Length() const { return sqrtf(x * x + y * y); }                 // b2math.d:142-145
    f32 LengthSquared() const { return x * x + y * y; }
    f32 Normalize() {                                                   // b2math.d:160-175
        f32 length = Length();
        if (length < kEpsilon) return 0.0f;
        f32 invLength = 1.0f / length;
        x *= invLength;
        y *= invLength;
        return length;
    }
};
static inline Vec2 operator+(Vec2 a, Vec2 b) { return Vec2(a.x + b.x, a.y + b.y); }
static inline Vec2 operator-(Vec2 a, Vec2 b) { return Vec2(a.x - b.x, a.y - b.y); }
// scalar * vector: b2Vec2.opBinary!"*"(float) computes s * x (b2math.d:106-116)
static inline Vec2 operator*(f32 s, Vec2 v) { return Vec2(s * v.x, s * v.y); }
static inline bool operator==(Vec2 a, Vec2 b) { return a.x == b.x && a.y == b.y; }

struct Vec3 {
    f32 x = 0, y = 0, z = 0;
    Vec3() {}
    Vec3(f32 a, f32 b, f32 c) : x(a), y(b), z(c) {}
    void SetZero() { x = 0.0f; y = 0.0f; z = 0.0f; }
    Vec3 operator-() const { return Vec3(-x, -y, -z); }
    void operator+=(Vec3 v) { x += v.x; y += v.y; z += v.z; }
    void operator*=(f32 s) { x *= s; y *= s; z *= s; }
};

static inline f32 Dot(Vec2 a, Vec2 b) { return a.x * b.x + a.y * b.y; }
static inline f32 Cross(Vec2 a, Vec2 b) { return a.x * b.y - a.y * b.x; }
static inline Vec2 Cross(Vec2 a, f32 s) { return Vec2(s * a.y, -s * a.x); }
static inline Vec2 Cross(f32 s, Vec2 a) { return Vec2(-s * a.y, s * a.x); }
static inline f32 Dot(Vec3 a, Vec3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
static inline Vec3 Cross(Vec3 a, Vec3 b) {
    return Vec3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
static inline f32 DistanceSquared(Vec2 a, Vec2 b) { Vec2 c = a - b; return Dot(c, c); }
static inline f32 Distance(Vec2 a, Vec2 b) { Vec2 c = a - b; return c.Length(); }

template <class T> static inline T Abs(T a) { return a > T(0) ? a : -a; }
template <class T> static inline T Min(T a, T b) { return a < b ? a : b; }
template <class T> static inline T Max(T a, T b) { return a > b ? a : b; }
static inline Vec2 Min(Vec2 a, Vec2 b) { return Vec2(Min(a.x, b.x), Min(a.y, b.y)); }
static inline Vec2 Max(Vec2 a, Vec2 b) { return Vec2(Max(a.x, b.x), Max(a.y, b.y)); }
template <class T> static inline T Clamp(T a, T low, T high) { return Max(low, Min(a, high)); }

struct Mat22 {                                                          // b2math.d:276-361
    Vec2 ex, ey;
    void SetZero() { ex.SetZero(); ey.SetZero(); }
    Mat22 GetInverse() const {
        f32 a = ex.x, b = ey.x, c = ex.y, d = ey.y;
        Mat22 B;
        f32 det = a * d - b * c;
        if (det != 0.0f) det = 1.0f / det;
        B.ex.x = det * d;
        B.ey.x = -det * b;
        B.ex.y = -det * c;
        B.ey.y = det * a;
        return B;
    }
    Vec2 Solve(Vec2 b) const {
        f32 a11 = ex.x, a12 = ey.x, a21 = ex.y, a22 = ey.y;
        f32 det = a11 * a22 - a12 * a21;
        if (det != 0.0f) det = 1.0f / det;
        Vec2 x;
        x.x = det * (a22 * b.x - a12 * b.y);
        x.y = det * (a11 * b.y - a21 * b.x);
        return x;
    }
};
static inline Vec2 Mul(const Mat22& A, Vec2 v) {
    return Vec2(A.ex.x * v.x + A.ey.x * v.y, A.ex.y * v.x + A.ey.y * v.y);
}

struct Mat33 {                                                          // b2math.d:364-466
    Vec3 ex, ey, ez;
    Vec3 Solve33(Vec3 b) const {
        f32 det = Dot(ex, Cross(ey, ez));
        if (det != 0.0f) det = 1.0f / det;
        Vec3 x;
        x.x = det * Dot(b, Cross(ey, ez));
        x.y = det * Dot(ex, Cross(b, ez));
        x.z = det * Dot(ex, Cross(ey, b));
        return x;
    }
    void GetInverse22(Mat33* M) const {                                 // b2math.d:419-440
        f32 a = ex.x, b = ey.x, c = ex.y, d = ey.y;
        f32 det = a * d - b * c;
        if (det != 0.0f) det = 1.0f / det;
        M->ex.x = det * d;
        M->ey.x = -det * b;
        M->ex.z = 0.0f;
        M->ex.y = -det * c;
        M->ey.y = det * a;
        M->ey.z = 0.0f;
        M->ez.x = 0.0f;
        M->ez.y = 0.0f;
        M->ez.z = 0.0f;
    }
    void GetSymInverse33(Mat33* M) const {                              // b2math.d:442-465
        f32 det = Dot(ex, Cross(ey, ez));
        if (det != 0.0f) det = 1.0f / det;
        f32 a11 = ex.x, a12 = ey.x, a13 = ez.x;
        f32 a22 = ey.y, a23 = ez.y;
        f32 a33 = ez.z;
        M->ex.x = det * (a22 * a33 - a23 * a23);
        M->ex.y = det * (a13 * a23 - a12 * a33);
        M->ex.z = det * (a12 * a23 - a13 * a22);
        M->ey.x = M->ex.y;
        M->ey.y = det * (a11 * a33 - a13 * a13);
        M->ey.z = det * (a13 * a12 - a11 * a23);
        M->ez.x = M->ex.z;
        M->ez.y = M->ey.z;
        M->ez.z = det * (a11 * a22 - a12 * a12);
    }
    Vec2 Solve22(Vec2 b) const {
        f32 a11 = ex.x, a12 = ey.x, a21 = ex.y, a22 = ey.y;
        f32 det = a11 * a22 - a12 * a21;
        if (det != 0.0f) det = 1.0f / det;
        Vec2 x;
        x.x = det * (a22 * b.x - a12 * b.y);
        x.y = det * (a11 * b.y - a21 * b.x);
        return x;
    }
};
static inline Vec3 Mul(const Mat33& A, Vec3 v) {                        // b2math.d:679-682
    return Vec3((v.x * A.ex.x + v.y * A.ey.x) + v.z * A.ez.x, (v.x * A.ex.y + v.y * A.ey.y) + v.z * A.ez.y,
                (v.x * A.ex.z + v.y * A.ey.z) + v.z * A.ez.z);
}
static inline Vec2 Mul22(const Mat33& A, Vec2 v) {                      // b2math.d:685-688
    return Vec2(A.ex.x * v.x + A.ey.x * v.y, A.ex.y * v.x + A.ey.y * v.y);
}

static inline void SinCos(f32 angle, f32* s, f32* c) {
    if (g_trig_mode == 0) {
        *s = ::sinf(angle);
        *c = ::cosf(angle);
    } else {
        dbox_sincosf(angle, s, c);
    }
}

struct Rot {                                                            // b2math.d:469-521
    f32 s = 0, c = 0;
    Rot() {}
    explicit Rot(f32 angle) { Set(angle); }
    void Set(f32 angle) { SinCos(angle, &s, &c); }
    void SetIdentity() { s = 0.0f; c = 1.0f; }
};
static inline Vec2 Mul(Rot q, Vec2 v) { return Vec2(q.c * v.x - q.s * v.y, q.s * v.x + q.c * v.y); }
static inline Vec2 MulT(Rot q, Vec2 v) { return Vec2(q.c * v.x + q.s * v.y, -q.s * v.x + q.c * v.y); }
static inline Rot MulT(Rot q, Rot r) {                                  // b2math.d:708-719
    Rot qr;
    qr.s = q.c * r.s - q.s * r.c;
    qr.c = q.c * r.c + q.s * r.s;
    return qr;
}

struct Transform {                                                      // b2math.d:525-551
    Vec2 p;
    Rot q;
    void SetIdentity() { p.SetZero(); q.SetIdentity(); }
};
static inline Vec2 Mul(const Transform& T, Vec2 v) {                    // b2math.d:734-740
    f32 x = (T.q.c * v.x - T.q.s * v.y) + T.p.x;
    f32 y = (T.q.s * v.x + T.q.c * v.y) + T.p.y;
    return Vec2(x, y);
}
static inline Vec2 MulT(const Transform& T, Vec2 v) {                   // b2math.d:743-751
    f32 px = v.x - T.p.x;
    f32 py = v.y - T.p.y;
    f32 x = (T.q.c * px + T.q.s * py);
    f32 y = (-T.q.s * px + T.q.c * py);
    return Vec2(x, y);
}
static inline Transform MulT(const Transform& A, const Transform& B) {  // b2math.d:764-770
    Transform C;
    C.q = MulT(A.q, B.q);
    C.p = MulT(A.q, B.p - A.p);
    return C;
}

struct Sweep {                                                          // b2math.d:554-593
    Vec2 localCenter;
    Vec2 c0, c;
    f32 a0 = 0, a = 0;
    f32 alpha0 = 0;
    void GetTransform(Transform* xf, f32 beta) const {
        xf->p = (1.0f - beta) * c0 + beta * c;
        f32 angle = (1.0f - beta) * a0 + beta * a;
        xf->q.Set(angle);
        xf->p -= Mul(xf->q, localCenter);
    }
    void Advance(f32 alpha) {
        f32 beta = (alpha - alpha0) / (1.0f - alpha0);
        c0 += beta * (c - c0);
        a0 += beta * (a - a0);
        alpha0 = alpha;
    }
    void Normalize() {
        f32 twoPi = 2.0f * kPi;
        f32 d = twoPi * floorf(a0 / twoPi);
        a0 -= d;
        a -= d;
    }
};

// ------------------------------------------------------------ shapes
enum { kCircle = 0, kEdge = 1, kPolygon = 2, kChain = 3 };

struct Shape {
    int type = kCircle;
    f32 radius = 0;
    Vec2 p;                       // circle center (b2circleshape.d:157)
    Vec2 centroid;                // polygon (b2polygonshape.d:561-565)
    Vec2 vertices[kMaxPolygonVertices];
    Vec2 normals[kMaxPolygonVertices];
    int count = 0;
    // edge (b2edgeshape.d): vertices[0..1] = m_vertex1, m_vertex2 (count 2); ghost vertices
    Vec2 vertex0, vertex3;
    bool hasVertex0 = false, hasVertex3 = false;
};

struct MassData { f32 mass = 0; Vec2 center; f32 I = 0; };

struct AABB {
    Vec2 lowerBound, upperBound;
    f32 GetPerimeter() const {                                          // b2collision.d:306-311
        f32 wx = upperBound.x - lowerBound.x;
        f32 wy = upperBound.y - lowerBound.y;
        return 2.0f * (wx + wy);
    }
    void Combine(const AABB& a) { lowerBound = Min(lowerBound, a.lowerBound); upperBound = Max(upperBound, a.upperBound); }
    void Combine(const AABB& a, const AABB& b) {
        lowerBound = Min(a.lowerBound, b.lowerBound);
        upperBound = Max(a.upperBound, b.upperBound);
    }
    bool Contains(const AABB& aabb) const {                             // b2collision.d:329-337
        bool result = true;
        result = result && lowerBound.x <= aabb.lowerBound.x;
        result = result && lowerBound.y <= aabb.lowerBound.y;
        result = result && aabb.upperBound.x <= upperBound.x;
        result = result && aabb.upperBound.y <= upperBound.y;
        return result;
    }
};

static inline bool TestOverlap(const AABB& a, const AABB& b) {          // b2collision.d:470-483
    Vec2 d1, d2;
    d1 = b.lowerBound - a.upperBound;
    d2 = a.lowerBound - b.upperBound;
    if (d1.x > 0.0f || d1.y > 0.0f) return false;
    if (d2.x > 0.0f || d2.y > 0.0f) return false;
    return true;
}

static Vec2 ComputeCentroid(const Vec2* vs, int count) {                // b2polygonshape.d:506-554
    Vec2 c;
    c.Set(0.0f, 0.0f);
    f32 area = 0.0f;
    Vec2 pRef(0.0f, 0.0f);
    const f32 inv3 = 1.0f / 3.0f;
    for (int i = 0; i < count; ++i) {
        Vec2 p1 = pRef;
        Vec2 p2 = vs[i];
        Vec2 p3 = i + 1 < count ? vs[i + 1] : vs[0];
        Vec2 e1 = p2 - p1;
        Vec2 e2 = p3 - p1;
        f32 D = Cross(e1, e2);
        f32 triangleArea = 0.5f * D;
        area += triangleArea;
        c += (triangleArea * inv3) * ((p1 + p2) + p3);
    }
    c *= 1.0f / area;
    return c;
}

static void PolygonSetAsBox(Shape* s, f32 hx, f32 hy) {                 // b2polygonshape.d:220-232
    s->count = 4;
    s->vertices[0].Set(-hx, -hy);
    s->vertices[1].Set(hx, -hy);
    s->vertices[2].Set(hx, hy);
    s->vertices[3].Set(-hx, hy);
    s->normals[0].Set(0.0f, -1.0f);
    s->normals[1].Set(1.0f, 0.0f);
    s->normals[2].Set(0.0f, 1.0f);
    s->normals[3].Set(-1.0f, 0.0f);
    s->centroid.SetZero();
}

static void PolygonSetAsBox(Shape* s, f32 hx, f32 hy, Vec2 center, f32 angle) {  // b2polygonshape.d:238-262
    PolygonSetAsBox(s, hx, hy);
    s->centroid = center;
    Transform xf;
    xf.p = center;
    xf.q.Set(angle);
    for (int i = 0; i < s->count; ++i) {
        s->vertices[i] = Mul(xf, s->vertices[i]);
        s->normals[i] = Mul(xf.q, s->normals[i]);
    }
}

// b2PolygonShape.Set: weld, gift-wrap hull, normals, centroid (b2polygonshape.d:74-209).
// Returns false for degenerate input (the reference asserts).
static bool PolygonSet(Shape* s, const Vec2* vertices, int count) {
    if (count < 3) { PolygonSetAsBox(s, 1.0f, 1.0f); return false; }
    int n = Min(count, kMaxPolygonVertices);
    Vec2 ps[kMaxPolygonVertices];
    int tempCount = 0;
    for (int i = 0; i < n; ++i) {
        Vec2 v = vertices[i];
        bool unique = true;
        for (int j = 0; j < tempCount; ++j) {
            if (DistanceSquared(v, ps[j]) < 0.5f * kLinearSlop) { unique = false; break; }
        }
        if (unique) ps[tempCount++] = v;
    }
    n = tempCount;
    if (n < 3) { PolygonSetAsBox(s, 1.0f, 1.0f); return false; }
    int i0 = 0;
    f32 x0 = ps[0].x;
    for (int i = 1; i < n; ++i) {
        f32 x = ps[i].x;
        if (x > x0 || (x == x0 && ps[i].y < ps[i0].y)) { i0 = i; x0 = x; }
    }
    int hull[kMaxPolygonVertices];
    int m = 0;
    int ih = i0;
    for (;;) {
        if (m >= kMaxPolygonVertices) { PolygonSetAsBox(s, 1.0f, 1.0f); return false; }
        hull[m] = ih;
        int ie = 0;
        for (int j = 1; j < n; ++j) {
            if (ie == ih) { ie = j; continue; }
            Vec2 r = ps[ie] - ps[hull[m]];
            Vec2 v = ps[j] - ps[hull[m]];
            f32 c = Cross(r, v);
            if (c < 0.0f) ie = j;
            if (c == 0.0f && v.LengthSquared() > r.LengthSquared()) ie = j;
        }
        ++m;
        ih = ie;
        if (ie == i0) break;
    }
    if (m < 3) { PolygonSetAsBox(s, 1.0f, 1.0f); return false; }
    s->count = m;
    for (int i = 0; i < m; ++i) s->vertices[i] = ps[hull[i]];
    for (int i = 0; i < m; ++i) {
        int i1 = i;
        int i2 = i + 1 < m ? i + 1 : 0;
        Vec2 edge = s->vertices[i2] - s->vertices[i1];
        s->normals[i] = Cross(edge, 1.0f);
        s->normals[i].Normalize();
    }
    s->centroid = ComputeCentroid(s->vertices, m);
    return true;
}

static void ShapeComputeAABB(const Shape& s, AABB* aabb, const Transform& xf) {
    if (s.type == kCircle) {                                            // b2circleshape.d:110-117
        Vec2 p = xf.p + Mul(xf.q, s.p);
        aabb->lowerBound.Set(p.x - s.radius, p.y - s.radius);
        aabb->upperBound.Set(p.x + s.radius, p.y + s.radius);
        return;
    }
    Vec2 lower = Mul(xf, s.vertices[0]);                                // b2polygonshape.d:356-373
    Vec2 upper = lower;
    for (int i = 1; i < s.count; ++i) {
        Vec2 v = Mul(xf, s.vertices[i]);
        lower = Min(lower, v);
        upper = Max(upper, v);
    }
    Vec2 r(s.radius, s.radius);
    aabb->lowerBound = lower - r;
    aabb->upperBound = upper + r;
}

static void ShapeComputeMass(const Shape& s, MassData* md, f32 density) {
    if (s.type == kEdge) {                                              // b2edgeshape.d: no mass
        md->mass = 0.0f;
        md->center = 0.5f * (s.vertices[0] + s.vertices[1]);
        md->I = 0.0f;
        return;
    }
    if (s.type == kCircle) {                                            // b2circleshape.d:120-127
        md->mass = ((density * kPi) * s.radius) * s.radius;
        md->center = s.p;
        md->I = md->mass * ((0.5f * s.radius) * s.radius + Dot(s.p, s.p));
        return;
    }
    Vec2 center;                                                        // b2polygonshape.d:376-459
    center.Set(0.0f, 0.0f);
    f32 area = 0.0f;
    f32 I = 0.0f;
    Vec2 sref(0.0f, 0.0f);
    for (int i = 0; i < s.count; ++i) sref += s.vertices[i];
    sref *= 1.0f / (f32)s.count;
    const f32 k_inv3 = 1.0f / 3.0f;
    for (int i = 0; i < s.count; ++i) {
        Vec2 e1 = s.vertices[i] - sref;
        Vec2 e2 = i + 1 < s.count ? s.vertices[i + 1] - sref : s.vertices[0] - sref;
        f32 D = Cross(e1, e2);
        f32 triangleArea = 0.5f * D;
        area += triangleArea;
        center += (triangleArea * k_inv3) * (e1 + e2);
        f32 ex1 = e1.x, ey1 = e1.y;
        f32 ex2 = e2.x, ey2 = e2.y;
        f32 intx2 = (ex1 * ex1 + ex2 * ex1) + ex2 * ex2;
        f32 inty2 = (ey1 * ey1 + ey2 * ey1) + ey2 * ey2;
        I += ((0.25f * k_inv3) * D) * (intx2 + inty2);
    }
    md->mass = density * area;
    center *= 1.0f / area;
    md->center = center + sref;
    md->I = density * I;
    md->I += md->mass * (Dot(md->center, md->center) - Dot(center, center));
}

// ------------------------------------------------------------ manifolds
// collision/b2collision.d:38-114
union ContactID {
    struct { uint8_t indexA, indexB, typeA, typeB; } cf;
    uint32_t key;
};
enum { kFeatureVertex = 0, kFeatureFace = 1 };

struct ManifoldPoint {
    Vec2 localPoint;
    f32 normalImpulse = 0;
    f32 tangentImpulse = 0;
    ContactID id;
    ManifoldPoint() { id.key = 0; }
};

enum { kManifoldCircles = 0, kManifoldFaceA = 1, kManifoldFaceB = 2 };

struct Manifold {
    ManifoldPoint points[kMaxManifoldPoints];
    Vec2 localNormal;
    Vec2 localPoint;
    int type = kManifoldCircles;
    int pointCount = 0;
};

struct WorldManifold {                                                  // b2collision.d:117-196
    Vec2 normal;
    Vec2 points[kMaxManifoldPoints];
    f32 separations[kMaxManifoldPoints] = {0, 0};
    void Initialize(const Manifold* manifold, const Transform& xfA, f32 radiusA,
                    const Transform& xfB, f32 radiusB) {
        if (manifold->pointCount == 0) return;
        switch (manifold->type) {
        case kManifoldCircles: {
            normal.Set(1.0f, 0.0f);
            Vec2 pointA = Mul(xfA, manifold->localPoint);
            Vec2 pointB = Mul(xfB, manifold->points[0].localPoint);
            if (DistanceSquared(pointA, pointB) > kEpsilon * kEpsilon) {
                normal = pointB - pointA;
                normal.Normalize();
            }
            Vec2 cA = pointA + radiusA * normal;
            Vec2 cB = pointB - radiusB * normal;
            points[0] = 0.5f * (cA + cB);
            separations[0] = Dot(cB - cA, normal);
        } break;
        case kManifoldFaceA: {
            normal = Mul(xfA.q, manifold->localNormal);
            Vec2 planePoint = Mul(xfA, manifold->localPoint);
            for (int i = 0; i < manifold->pointCount; ++i) {
                Vec2 clipPoint = Mul(xfB, manifold->points[i].localPoint);
                Vec2 cA = clipPoint + (radiusA - Dot(clipPoint - planePoint, normal)) * normal;
                Vec2 cB = clipPoint - radiusB * normal;
                points[i] = 0.5f * (cA + cB);
                separations[i] = Dot(cB - cA, normal);
            }
        } break;
        case kManifoldFaceB: {
            normal = Mul(xfB.q, manifold->localNormal);
            Vec2 planePoint = Mul(xfB, manifold->localPoint);
            for (int i = 0; i < manifold->pointCount; ++i) {
                Vec2 clipPoint = Mul(xfA, manifold->points[i].localPoint);
                Vec2 cB = clipPoint + (radiusB - Dot(clipPoint - planePoint, normal)) * normal;
                Vec2 cA = clipPoint - radiusA * normal;
                points[i] = 0.5f * (cA + cB);
                separations[i] = Dot(cA - cB, normal);
            }
            normal = -normal;
        } break;
        default: break;
        }
    }
};

struct ClipVertex { Vec2 v; ContactID id; ClipVertex() { id.key = 0; } };

static int ClipSegmentToLine(ClipVertex vOut[2], const ClipVertex vIn[2], Vec2 normal, f32 offset,
                             int vertexIndexA) {                        // b2collision.d:413-446
    int numOut = 0;
    f32 distance0 = Dot(normal, vIn[0].v) - offset;
    f32 distance1 = Dot(normal, vIn[1].v) - offset;
    if (distance0 <= 0.0f) vOut[numOut++] = vIn[0];
    if (distance1 <= 0.0f) vOut[numOut++] = vIn[1];
    if (distance0 * distance1 < 0.0f) {
        f32 interp = distance0 / (distance0 - distance1);
        vOut[numOut].v = vIn[0].v + interp * (vIn[1].v - vIn[0].v);
        vOut[numOut].id.cf.indexA = (uint8_t)vertexIndexA;
        vOut[numOut].id.cf.indexB = vIn[0].id.cf.indexB;
        vOut[numOut].id.cf.typeA = kFeatureVertex;
        vOut[numOut].id.cf.typeB = kFeatureFace;
        ++numOut;
    }
    return numOut;
}

// collision/b2collidepolygon.d:29-71
static f32 FindMaxSeparation(int* edgeIndex, const Shape& poly1, const Transform& xf1,
                             const Shape& poly2, const Transform& xf2) {
    int count1 = poly1.count;
    int count2 = poly2.count;
    const Vec2* n1s = poly1.normals;
    const Vec2* v1s = poly1.vertices;
    const Vec2* v2s = poly2.vertices;
    Transform xf = MulT(xf2, xf1);
    int bestIndex = 0;
    f32 maxSeparation = -kMaxFloat;
    for (int i = 0; i < count1; ++i) {
        Vec2 n = Mul(xf.q, n1s[i]);
        Vec2 v1 = Mul(xf, v1s[i]);
        f32 si = kMaxFloat;
        for (int j = 0; j < count2; ++j) {
            f32 sij = Dot(n, v2s[j] - v1);
            if (sij < si) si = sij;
        }
        if (si > maxSeparation) { maxSeparation = si; bestIndex = i; }
    }
    *edgeIndex = bestIndex;
    return maxSeparation;
}

// collision/b2collidepolygon.d:73-118
static void FindIncidentEdge(ClipVertex c[2], const Shape& poly1, const Transform& xf1, int edge1,
                             const Shape& poly2, const Transform& xf2) {
    const Vec2* normals1 = poly1.normals;
    int count2 = poly2.count;
    const Vec2* vertices2 = poly2.vertices;
    const Vec2* normals2 = poly2.normals;
    Vec2 normal1 = MulT(xf2.q, Mul(xf1.q, normals1[edge1]));
    int index = 0;
    f32 minDot = kMaxFloat;
    for (int i = 0; i < count2; ++i) {
        f32 dot = Dot(normal1, normals2[i]);
        if (dot < minDot) { minDot = dot; index = i; }
    }
    int i1 = index;
    int i2 = i1 + 1 < count2 ? i1 + 1 : 0;
    c[0].v = Mul(xf2, vertices2[i1]);
    c[0].id.cf.indexA = (uint8_t)edge1;
    c[0].id.cf.indexB = (uint8_t)i1;
    c[0].id.cf.typeA = kFeatureFace;
    c[0].id.cf.typeB = kFeatureVertex;
    c[1].v = Mul(xf2, vertices2[i2]);
    c[1].id.cf.indexA = (uint8_t)edge1;
    c[1].id.cf.indexB = (uint8_t)i2;
    c[1].id.cf.typeA = kFeatureFace;
    c[1].id.cf.typeB = kFeatureVertex;
}

// collision/b2collidepolygon.d:127-254
static void CollidePolygons(Manifold* manifold, const Shape& polyA, const Transform& xfA,
                            const Shape& polyB, const Transform& xfB) {
    manifold->pointCount = 0;
    f32 totalRadius = polyA.radius + polyB.radius;
    int edgeA = 0;
    f32 separationA = FindMaxSeparation(&edgeA, polyA, xfA, polyB, xfB);
    if (separationA > totalRadius) return;
    int edgeB = 0;
    f32 separationB = FindMaxSeparation(&edgeB, polyB, xfB, polyA, xfA);
    if (separationB > totalRadius) return;
    const Shape* poly1;
    const Shape* poly2;
    Transform xf1, xf2;
    int edge1;
    uint8_t flip;
    const f32 k_tol = 0.1f * kLinearSlop;
    if (separationB > separationA + k_tol) {
        poly1 = &polyB; poly2 = &polyA; xf1 = xfB; xf2 = xfA; edge1 = edgeB;
        manifold->type = kManifoldFaceB;
        flip = 1;
    } else {
        poly1 = &polyA; poly2 = &polyB; xf1 = xfA; xf2 = xfB; edge1 = edgeA;
        manifold->type = kManifoldFaceA;
        flip = 0;
    }
    ClipVertex incidentEdge[2];
    FindIncidentEdge(incidentEdge, *poly1, xf1, edge1, *poly2, xf2);
    int count1 = poly1->count;
    const Vec2* vertices1 = poly1->vertices;
    int iv1 = edge1;
    int iv2 = edge1 + 1 < count1 ? edge1 + 1 : 0;
    Vec2 v11 = vertices1[iv1];
    Vec2 v12 = vertices1[iv2];
    Vec2 localTangent = v12 - v11;
    localTangent.Normalize();
    Vec2 localNormal = Cross(localTangent, 1.0f);
    Vec2 planePoint = 0.5f * (v11 + v12);
    Vec2 tangent = Mul(xf1.q, localTangent);
    Vec2 normal = Cross(tangent, 1.0f);
    v11 = Mul(xf1, v11);
    v12 = Mul(xf1, v12);
    f32 frontOffset = Dot(normal, v11);
    f32 sideOffset1 = -Dot(tangent, v11) + totalRadius;
    f32 sideOffset2 = Dot(tangent, v12) + totalRadius;
    ClipVertex clipPoints1[2];
    ClipVertex clipPoints2[2];
    int np = ClipSegmentToLine(clipPoints1, incidentEdge, -tangent, sideOffset1, iv1);
    if (np < 2) return;
    np = ClipSegmentToLine(clipPoints2, clipPoints1, tangent, sideOffset2, iv2);
    if (np < 2) return;
    manifold->localNormal = localNormal;
    manifold->localPoint = planePoint;
    int pointCount = 0;
    for (int i = 0; i < kMaxManifoldPoints; ++i) {
        f32 separation = Dot(normal, clipPoints2[i].v) - frontOffset;
        if (separation <= totalRadius) {
            ManifoldPoint* cp = manifold->points + pointCount;
            cp->localPoint = MulT(xf2, clipPoints2[i].v);
            cp->id = clipPoints2[i].id;
            if (flip) {
                ContactID cf = cp->id;
                cp->id.cf.indexA = cf.cf.indexB;
                cp->id.cf.indexB = cf.cf.indexA;
                cp->id.cf.typeA = cf.cf.typeB;
                cp->id.cf.typeB = cf.cf.typeA;
            }
            ++pointCount;
        }
    }
    manifold->pointCount = pointCount;
}

// collision/b2collidecircle.d:29-56
static void CollideCircles(Manifold* manifold, const Shape& circleA, const Transform& xfA,
                           const Shape& circleB, const Transform& xfB) {
    manifold->pointCount = 0;
    Vec2 pA = Mul(xfA, circleA.p);
    Vec2 pB = Mul(xfB, circleB.p);
    Vec2 d = pB - pA;
    f32 distSqr = Dot(d, d);
    f32 rA = circleA.radius, rB = circleB.radius;
    f32 radius = rA + rB;
    if (distSqr > radius * radius) return;
    manifold->type = kManifoldCircles;
    manifold->localPoint = circleA.p;
    manifold->localNormal.SetZero();
    manifold->pointCount = 1;
    manifold->points[0].localPoint = circleB.p;
    manifold->points[0].id.key = 0;
}

// collision/b2collidecircle.d:59-164
static void CollidePolygonAndCircle(Manifold* manifold, const Shape& polygonA, const Transform& xfA,
                                    const Shape& circleB, const Transform& xfB) {
    manifold->pointCount = 0;
    Vec2 c = Mul(xfB, circleB.p);
    Vec2 cLocal = MulT(xfA, c);
    int normalIndex = 0;
    f32 separation = -kMaxFloat;
    f32 radius = polygonA.radius + circleB.radius;
    int vertexCount = polygonA.count;
    const Vec2* vertices = polygonA.vertices;
    const Vec2* normals = polygonA.normals;
    for (int i = 0; i < vertexCount; ++i) {
        f32 s = Dot(normals[i], cLocal - vertices[i]);
        if (s > radius) return;
        if (s > separation) { separation = s; normalIndex = i; }
    }
    int vertIndex1 = normalIndex;
    int vertIndex2 = vertIndex1 + 1 < vertexCount ? vertIndex1 + 1 : 0;
    Vec2 v1 = vertices[vertIndex1];
    Vec2 v2 = vertices[vertIndex2];
    if (separation < kEpsilon) {
        manifold->pointCount = 1;
        manifold->type = kManifoldFaceA;
        manifold->localNormal = normals[normalIndex];
        manifold->localPoint = 0.5f * (v1 + v2);
        manifold->points[0].localPoint = circleB.p;
        manifold->points[0].id.key = 0;
        return;
    }
    f32 u1 = Dot(cLocal - v1, v2 - v1);
    f32 u2 = Dot(cLocal - v2, v1 - v2);
    if (u1 <= 0.0f) {
        if (DistanceSquared(cLocal, v1) > radius * radius) return;
        manifold->pointCount = 1;
        manifold->type = kManifoldFaceA;
        manifold->localNormal = cLocal - v1;
        manifold->localNormal.Normalize();
        manifold->localPoint = v1;
        manifold->points[0].localPoint = circleB.p;
        manifold->points[0].id.key = 0;
    } else if (u2 <= 0.0f) {
        if (DistanceSquared(cLocal, v2) > radius * radius) return;
        manifold->pointCount = 1;
        manifold->type = kManifoldFaceA;
        manifold->localNormal = cLocal - v2;
        manifold->localNormal.Normalize();
        manifold->localPoint = v2;
        manifold->points[0].localPoint = circleB.p;
        manifold->points[0].id.key = 0;
    } else {
        Vec2 faceCenter = 0.5f * (v1 + v2);
        f32 separation2 = Dot(cLocal - faceCenter, normals[vertIndex1]);
        if (separation2 > radius) return;
        manifold->pointCount = 1;
        manifold->type = kManifoldFaceA;
        manifold->localNormal = normals[vertIndex1];
        manifold->localPoint = faceCenter;
        manifold->points[0].localPoint = circleB.p;
        manifold->points[0].id.key = 0;
    }
}

// b2CollideEdgeAndCircle (b2collideedge.d:31-155): the circle against the edge's regions A, B
// (vertices, unless an adjacent edge owns the region) and AB (the face)
static void CollideEdgeAndCircle(Manifold* manifold, const Shape& edgeA, const Transform& xfA,
                                 const Shape& circleB, const Transform& xfB) {
    manifold->pointCount = 0;
    Vec2 Q = MulT(xfA, Mul(xfB, circleB.p));                            // circle in the edge's frame
    Vec2 A = edgeA.vertices[0], B = edgeA.vertices[1];
    Vec2 e = B - A;
    f32 u = Dot(e, B - Q);                                              // barycentric coordinates
    f32 v = Dot(e, Q - A);
    f32 radius = edgeA.radius + circleB.radius;
    ContactID id;
    id.key = 0;
    id.cf.indexB = 0;
    id.cf.typeB = kFeatureVertex;
    if (v <= 0.0f) {                                                    // region A
        Vec2 P = A;
        Vec2 d = Q - P;
        f32 dd = Dot(d, d);
        if (dd > radius * radius) return;
        if (edgeA.hasVertex0) {
            Vec2 A1 = edgeA.vertex0;
            Vec2 B1 = A;
            Vec2 e1 = B1 - A1;
            f32 u1 = Dot(e1, B1 - Q);
            if (u1 > 0.0f) return;                                      // region AB of the previous edge
        }
        id.cf.indexA = 0;
        id.cf.typeA = kFeatureVertex;
        manifold->pointCount = 1;
        manifold->type = kManifoldCircles;
        manifold->localNormal.SetZero();
        manifold->localPoint = P;
        manifold->points[0].id = id;
        manifold->points[0].localPoint = circleB.p;
        return;
    }
    if (u <= 0.0f) {                                                    // region B
        Vec2 P = B;
        Vec2 d = Q - P;
        f32 dd = Dot(d, d);
        if (dd > radius * radius) return;
        if (edgeA.hasVertex3) {
            Vec2 B2 = edgeA.vertex3;
            Vec2 A2 = B;
            Vec2 e2 = B2 - A2;
            f32 v2 = Dot(e2, Q - A2);
            if (v2 > 0.0f) return;                                      // region AB of the next edge
        }
        id.cf.indexA = 1;
        id.cf.typeA = kFeatureVertex;
        manifold->pointCount = 1;
        manifold->type = kManifoldCircles;
        manifold->localNormal.SetZero();
        manifold->localPoint = P;
        manifold->points[0].id = id;
        manifold->points[0].localPoint = circleB.p;
        return;
    }
    f32 den = Dot(e, e);                                                // region AB
    Vec2 P = (1.0f / den) * (u * A + v * B);
    Vec2 d = Q - P;
    f32 dd = Dot(d, d);
    if (dd > radius * radius) return;
    Vec2 n(-e.y, e.x);
    if (Dot(n, Q - A) < 0.0f) n.Set(-n.x, -n.y);
    n.Normalize();
    id.cf.indexA = 0;
    id.cf.typeA = kFeatureFace;
    manifold->pointCount = 1;
    manifold->type = kManifoldFaceA;
    manifold->localNormal = n;
    manifold->localPoint = A;
    manifold->points[0].id = id;
    manifold->points[0].localPoint = circleB.p;
}

// b2EPCollider (b2collideedge.d:157-717): an edge against a polygon with the edge's
// adjacency (ghost vertices) limiting the admissible normals
struct EPCollider {
    enum { kUnknown = 0, kEdgeA, kEdgeB };
    struct Axis { int type = kUnknown; int index = 0; f32 separation = 0; };
    struct ReferenceFace { int i1 = 0, i2 = 0; Vec2 v1, v2, normal, sideNormal1, sideNormal2; f32 sideOffset1 = 0, sideOffset2 = 0; };
    Vec2 pv[kMaxPolygonVertices], pn[kMaxPolygonVertices];            // polygon B in frame A
    int pcount = 0;
    Transform xf;
    Vec2 centroidB, v0, v1, v2, v3, normal0, normal1, normal2, normal, lowerLimit, upperLimit;
    f32 radius = 0;
    bool front = false;

    Axis ComputeEdgeSeparation() const {                                // b2collideedge.d:636-653
        Axis axis;
        axis.type = kEdgeA;
        axis.index = front ? 0 : 1;
        axis.separation = kMaxFloat;
        for (int i = 0; i < pcount; ++i) {
            f32 s = Dot(normal, pv[i] - v1);
            if (s < axis.separation) axis.separation = s;
        }
        return axis;
    }

    Axis ComputePolygonSeparation() const {                             // b2collideedge.d:655-700
        Axis axis;
        axis.type = kUnknown;
        axis.index = -1;
        axis.separation = -kMaxFloat;
        Vec2 perp(-normal.y, normal.x);
        for (int i = 0; i < pcount; ++i) {
            Vec2 n = -pn[i];
            f32 s1 = Dot(n, pv[i] - v1);
            f32 s2 = Dot(n, pv[i] - v2);
            f32 s = Min(s1, s2);
            if (s > radius) {                                           // no collision
                axis.type = kEdgeB;
                axis.index = i;
                axis.separation = s;
                return axis;
            }
            if (Dot(n, perp) >= 0.0f) {                                 // adjacency
                if (Dot(n - upperLimit, normal) < -kAngularSlop) continue;
            } else {
                if (Dot(n - lowerLimit, normal) < -kAngularSlop) continue;
            }
            if (s > axis.separation) {
                axis.type = kEdgeB;
                axis.index = i;
                axis.separation = s;
            }
        }
        return axis;
    }

    void Collide(Manifold* manifold, const Shape& edgeA, const Transform& xfA, const Shape& polygonB,
                 const Transform& xfB) {                                // b2collideedge.d:193-634
        xf = MulT(xfA, xfB);
        centroidB = Mul(xf, polygonB.centroid);
        v0 = edgeA.vertex0;
        v1 = edgeA.vertices[0];
        v2 = edgeA.vertices[1];
        v3 = edgeA.vertex3;
        bool hasVertex0 = edgeA.hasVertex0, hasVertex3 = edgeA.hasVertex3;
        Vec2 edge1 = v2 - v1;
        edge1.Normalize();
        normal1.Set(edge1.y, -edge1.x);
        f32 offset1 = Dot(normal1, centroidB - v1);
        f32 offset0 = 0.0f, offset2 = 0.0f;
        bool convex1 = false, convex2 = false;
        if (hasVertex0) {                                               // a preceding edge
            Vec2 edge0 = v1 - v0;
            edge0.Normalize();
            normal0.Set(edge0.y, -edge0.x);
            convex1 = Cross(edge0, edge1) >= 0.0f;
            offset0 = Dot(normal0, centroidB - v0);
        }
        if (hasVertex3) {                                               // a following edge
            Vec2 edge2 = v3 - v2;
            edge2.Normalize();
            normal2.Set(edge2.y, -edge2.x);
            convex2 = Cross(edge1, edge2) > 0.0f;
            offset2 = Dot(normal2, centroidB - v2);
        }
        // front or back collision; the collision normal's limits
        auto set = [&](bool f, Vec2 nf, Vec2 lf, Vec2 uf, Vec2 nb, Vec2 lb, Vec2 ub) {
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
        pcount = polygonB.count;                                        // polygon B in frame A
        for (int i = 0; i < polygonB.count; ++i) {
            pv[i] = Mul(xf, polygonB.vertices[i]);
            pn[i] = Mul(xf.q, polygonB.normals[i]);
        }
        radius = 2.0f * kPolygonRadius;
        manifold->pointCount = 0;
        Axis edgeAxis = ComputeEdgeSeparation();
        if (edgeAxis.type == kUnknown) return;                          // no valid normal
        if (edgeAxis.separation > radius) return;
        Axis polygonAxis = ComputePolygonSeparation();
        if (polygonAxis.type != kUnknown && polygonAxis.separation > radius) return;
        const f32 k_relativeTol = 0.98f, k_absoluteTol = 0.001f;          // hysteresis
        Axis primaryAxis;
        if (polygonAxis.type == kUnknown) primaryAxis = edgeAxis;
        else if (polygonAxis.separation > k_relativeTol * edgeAxis.separation + k_absoluteTol) primaryAxis = polygonAxis;
        else primaryAxis = edgeAxis;
        ClipVertex ie[2];
        ReferenceFace rf;
        if (primaryAxis.type == kEdgeA) {
            manifold->type = kManifoldFaceA;
            int bestIndex = 0;                                          // the most anti-parallel polygon normal
            f32 bestValue = Dot(normal, pn[0]);
            for (int i = 1; i < pcount; ++i) {
                f32 value = Dot(normal, pn[i]);
                if (value < bestValue) { bestValue = value; bestIndex = i; }
            }
            int i1 = bestIndex;
            int i2 = i1 + 1 < pcount ? i1 + 1 : 0;
            ie[0].v = pv[i1];
            ie[0].id.cf.indexA = 0;
            ie[0].id.cf.indexB = (uint8_t)i1;
            ie[0].id.cf.typeA = kFeatureFace;
            ie[0].id.cf.typeB = kFeatureVertex;
            ie[1].v = pv[i2];
            ie[1].id.cf.indexA = 0;
            ie[1].id.cf.indexB = (uint8_t)i2;
            ie[1].id.cf.typeA = kFeatureFace;
            ie[1].id.cf.typeB = kFeatureVertex;
            if (front) { rf.i1 = 0; rf.i2 = 1; rf.v1 = v1; rf.v2 = v2; rf.normal = normal1; }
            else { rf.i1 = 1; rf.i2 = 0; rf.v1 = v2; rf.v2 = v1; rf.normal = -normal1; }
        } else {
            manifold->type = kManifoldFaceB;
            ie[0].v = v1;
            ie[0].id.cf.indexA = 0;
            ie[0].id.cf.indexB = (uint8_t)primaryAxis.index;
            ie[0].id.cf.typeA = kFeatureVertex;
            ie[0].id.cf.typeB = kFeatureFace;
            ie[1].v = v2;
            ie[1].id.cf.indexA = 0;
            ie[1].id.cf.indexB = (uint8_t)primaryAxis.index;
            ie[1].id.cf.typeA = kFeatureVertex;
            ie[1].id.cf.typeB = kFeatureFace;
            rf.i1 = primaryAxis.index;
            rf.i2 = rf.i1 + 1 < pcount ? rf.i1 + 1 : 0;
            rf.v1 = pv[rf.i1];
            rf.v2 = pv[rf.i2];
            rf.normal = pn[rf.i1];
        }
        rf.sideNormal1.Set(rf.normal.y, -rf.normal.x);
        rf.sideNormal2 = -rf.sideNormal1;
        rf.sideOffset1 = Dot(rf.sideNormal1, rf.v1);
        rf.sideOffset2 = Dot(rf.sideNormal2, rf.v2);
        ClipVertex clipPoints1[2], clipPoints2[2];                      // clip against the side edges
        int np = ClipSegmentToLine(clipPoints1, ie, rf.sideNormal1, rf.sideOffset1, rf.i1);
        if (np < kMaxManifoldPoints) return;
        np = ClipSegmentToLine(clipPoints2, clipPoints1, rf.sideNormal2, rf.sideOffset2, rf.i2);
        if (np < kMaxManifoldPoints) return;
        if (primaryAxis.type == kEdgeA) {
            manifold->localNormal = rf.normal;
            manifold->localPoint = rf.v1;
        } else {
            manifold->localNormal = polygonB.normals[rf.i1];
            manifold->localPoint = polygonB.vertices[rf.i1];
        }
        int pointCount = 0;
        for (int i = 0; i < kMaxManifoldPoints; ++i) {
            f32 separation = Dot(rf.normal, clipPoints2[i].v - rf.v1);
            if (separation <= radius) {
                ManifoldPoint* cp = manifold->points + pointCount;
                if (primaryAxis.type == kEdgeA) {
                    cp->localPoint = MulT(xf, clipPoints2[i].v);
                    cp->id = clipPoints2[i].id;
                } else {
                    cp->localPoint = clipPoints2[i].v;
                    cp->id.cf.typeA = clipPoints2[i].id.cf.typeB;
                    cp->id.cf.typeB = clipPoints2[i].id.cf.typeA;
                    cp->id.cf.indexA = clipPoints2[i].id.cf.indexB;
                    cp->id.cf.indexB = clipPoints2[i].id.cf.indexA;
                }
                ++pointCount;
            }
        }
        manifold->pointCount = pointCount;
    }
};

static void CollideEdgeAndPolygon(Manifold* manifold, const Shape& edgeA, const Transform& xfA,
                                  const Shape& polygonB, const Transform& xfB) {
    EPCollider collider;
    collider.Collide(manifold, edgeA, xfA, polygonB, xfB);
}

// ------------------------------------------------------------ distance (GJK)
// collision/b2distance.d
struct DistanceProxy {                                                  // b2distance.d:30-144
    const Vec2* vertices = nullptr;
    int count = 0;
    f32 radius = 0;
    void Set(const Shape& s) {
        if (s.type == kCircle) { vertices = &s.p; count = 1; radius = s.radius; }
        else { vertices = s.vertices; count = s.count; radius = s.radius; }
    }
    int GetSupport(Vec2 d) const {
        int bestIndex = 0;
        f32 bestValue = Dot(vertices[0], d);
        for (int i = 1; i < count; ++i) {
            f32 value = Dot(vertices[i], d);
            if (value > bestValue) { bestIndex = i; bestValue = value; }
        }
        return bestIndex;
    }
    Vec2 GetVertex(int index) const { return vertices[index]; }
};

struct SimplexCache { f32 metric = 0; uint16_t count = 0; uint8_t indexA[3] = {0, 0, 0}; uint8_t indexB[3] = {0, 0, 0}; };
struct DistanceInput { DistanceProxy proxyA, proxyB; Transform transformA, transformB; bool useRadii = false; };
struct DistanceOutput { Vec2 pointA, pointB; f32 distance = 0; int iterations = 0; };

struct SimplexVertex { Vec2 wA, wB, w; f32 a = 0; int indexA = 0, indexB = 0; };

struct Simplex {                                                        // b2distance.d:366-705
    SimplexVertex v[3];
    int count = 0;
    void ReadCache(const SimplexCache* cache, const DistanceProxy* proxyA, const Transform& transformA,
                   const DistanceProxy* proxyB, const Transform& transformB) {
        count = cache->count;
        for (int i = 0; i < count; ++i) {
            SimplexVertex* vv = v + i;
            vv->indexA = cache->indexA[i];
            vv->indexB = cache->indexB[i];
            Vec2 wALocal = proxyA->GetVertex(vv->indexA);
            Vec2 wBLocal = proxyB->GetVertex(vv->indexB);
            vv->wA = Mul(transformA, wALocal);
            vv->wB = Mul(transformB, wBLocal);
            vv->w = vv->wB - vv->wA;
            vv->a = 0.0f;
        }
        if (count > 1) {
            f32 metric1 = cache->metric;
            f32 metric2 = GetMetric();
            if (metric2 < 0.5f * metric1 || 2.0f * metric1 < metric2 || metric2 < kEpsilon) count = 0;
        }
        if (count == 0) {
            SimplexVertex* vv = v + 0;
            vv->indexA = 0;
            vv->indexB = 0;
            Vec2 wALocal = proxyA->GetVertex(0);
            Vec2 wBLocal = proxyB->GetVertex(0);
            vv->wA = Mul(transformA, wALocal);
            vv->wB = Mul(transformB, wBLocal);
            vv->w = vv->wB - vv->wA;
            vv->a = 1.0f;
            count = 1;
        }
    }
    void WriteCache(SimplexCache* cache) const {
        cache->metric = GetMetric();
        cache->count = (uint16_t)count;
        for (int i = 0; i < count; ++i) {
            cache->indexA[i] = (uint8_t)v[i].indexA;
            cache->indexB[i] = (uint8_t)v[i].indexB;
        }
    }
    Vec2 GetSearchDirection() const {
        if (count == 1) return -v[0].w;
        Vec2 e12 = v[1].w - v[0].w;
        f32 sgn = Cross(e12, -v[0].w);
        if (sgn > 0.0f) return Cross(1.0f, e12);
        return Cross(e12, 1.0f);
    }
    Vec2 GetClosestPoint() const {
        switch (count) {
        case 1: return v[0].w;
        case 2: return v[0].a * v[0].w + v[1].a * v[1].w;
        default: return Vec2(0.0f, 0.0f);
        }
    }
    void GetWitnessPoints(Vec2* pA, Vec2* pB) const {
        switch (count) {
        case 1: *pA = v[0].wA; *pB = v[0].wB; break;
        case 2:
            *pA = v[0].a * v[0].wA + v[1].a * v[1].wA;
            *pB = v[0].a * v[0].wB + v[1].a * v[1].wB;
            break;
        case 3:
            *pA = (v[0].a * v[0].wA + v[1].a * v[1].wA) + v[2].a * v[2].wA;
            *pB = *pA;
            break;
        default: break;
        }
    }
    f32 GetMetric() const {
        switch (count) {
        case 1: return 0.0f;
        case 2: return Distance(v[0].w, v[1].w);
        case 3: return Cross(v[1].w - v[0].w, v[2].w - v[0].w);
        default: return 0.0f;
        }
    }
    void Solve2() {
        Vec2 w1 = v[0].w;
        Vec2 w2 = v[1].w;
        Vec2 e12 = w2 - w1;
        f32 d12_2 = -Dot(w1, e12);
        if (d12_2 <= 0.0f) { v[0].a = 1.0f; count = 1; return; }
        f32 d12_1 = Dot(w2, e12);
        if (d12_1 <= 0.0f) { v[1].a = 1.0f; count = 1; v[0] = v[1]; return; }
        f32 inv_d12 = 1.0f / (d12_1 + d12_2);
        v[0].a = d12_1 * inv_d12;
        v[1].a = d12_2 * inv_d12;
        count = 2;
    }
    void Solve3() {
        Vec2 w1 = v[0].w;
        Vec2 w2 = v[1].w;
        Vec2 w3 = v[2].w;
        Vec2 e12 = w2 - w1;
        f32 w1e12 = Dot(w1, e12);
        f32 w2e12 = Dot(w2, e12);
        f32 d12_1 = w2e12;
        f32 d12_2 = -w1e12;
        Vec2 e13 = w3 - w1;
        f32 w1e13 = Dot(w1, e13);
        f32 w3e13 = Dot(w3, e13);
        f32 d13_1 = w3e13;
        f32 d13_2 = -w1e13;
        Vec2 e23 = w3 - w2;
        f32 w2e23 = Dot(w2, e23);
        f32 w3e23 = Dot(w3, e23);
        f32 d23_1 = w3e23;
        f32 d23_2 = -w2e23;
        f32 n123 = Cross(e12, e13);
        f32 d123_1 = n123 * Cross(w2, w3);
        f32 d123_2 = n123 * Cross(w3, w1);
        f32 d123_3 = n123 * Cross(w1, w2);
        if (d12_2 <= 0.0f && d13_2 <= 0.0f) { v[0].a = 1.0f; count = 1; return; }
        if (d12_1 > 0.0f && d12_2 > 0.0f && d123_3 <= 0.0f) {
            f32 inv_d12 = 1.0f / (d12_1 + d12_2);
            v[0].a = d12_1 * inv_d12;
            v[1].a = d12_2 * inv_d12;
            count = 2;
            return;
        }
        if (d13_1 > 0.0f && d13_2 > 0.0f && d123_2 <= 0.0f) {
            f32 inv_d13 = 1.0f / (d13_1 + d13_2);
            v[0].a = d13_1 * inv_d13;
            v[2].a = d13_2 * inv_d13;
            count = 2;
            v[1] = v[2];
            return;
        }
        if (d12_1 <= 0.0f && d23_2 <= 0.0f) { v[1].a = 1.0f; count = 1; v[0] = v[1]; return; }
        if (d13_1 <= 0.0f && d23_1 <= 0.0f) { v[2].a = 1.0f; count = 1; v[0] = v[2]; return; }
        if (d23_1 > 0.0f && d23_2 > 0.0f && d123_1 <= 0.0f) {
            f32 inv_d23 = 1.0f / (d23_1 + d23_2);
            v[1].a = d23_1 * inv_d23;
            v[2].a = d23_2 * inv_d23;
            count = 2;
            v[0] = v[2];
            return;
        }
        f32 inv_d123 = 1.0f / ((d123_1 + d123_2) + d123_3);
        v[0].a = d123_1 * inv_d123;
        v[1].a = d123_2 * inv_d123;
        v[2].a = d123_3 * inv_d123;
        count = 3;
    }
};

// collision/b2distance.d:185-350
static void ComputeDistance(DistanceOutput* output, SimplexCache* cache, const DistanceInput* input) {
    const DistanceProxy* proxyA = &input->proxyA;
    const DistanceProxy* proxyB = &input->proxyB;
    Transform transformA = input->transformA;
    Transform transformB = input->transformB;
    Simplex simplex;
    simplex.ReadCache(cache, proxyA, transformA, proxyB, transformB);
    SimplexVertex* vertices = simplex.v;
    const int k_maxIters = 20;
    int saveA[3], saveB[3];
    int saveCount = 0;
    int iter = 0;
    while (iter < k_maxIters) {
        saveCount = simplex.count;
        for (int i = 0; i < saveCount; ++i) { saveA[i] = vertices[i].indexA; saveB[i] = vertices[i].indexB; }
        switch (simplex.count) {
        case 1: break;
        case 2: simplex.Solve2(); break;
        case 3: simplex.Solve3(); break;
        default: break;
        }
        if (simplex.count == 3) break;
        Vec2 d = simplex.GetSearchDirection();
        if (d.LengthSquared() < kEpsilon * kEpsilon) break;
        SimplexVertex* vertex = vertices + simplex.count;
        vertex->indexA = proxyA->GetSupport(MulT(transformA.q, -d));
        vertex->wA = Mul(transformA, proxyA->GetVertex(vertex->indexA));
        vertex->indexB = proxyB->GetSupport(MulT(transformB.q, d));
        vertex->wB = Mul(transformB, proxyB->GetVertex(vertex->indexB));
        vertex->w = vertex->wB - vertex->wA;
        ++iter;
        bool duplicate = false;
        for (int i = 0; i < saveCount; ++i) {
            if (vertex->indexA == saveA[i] && vertex->indexB == saveB[i]) { duplicate = true; break; }
        }
        if (duplicate) break;
        ++simplex.count;
    }
    simplex.GetWitnessPoints(&output->pointA, &output->pointB);
    output->distance = Distance(output->pointA, output->pointB);
    output->iterations = iter;
    simplex.WriteCache(cache);
    if (input->useRadii) {
        f32 rA = proxyA->radius;
        f32 rB = proxyB->radius;
        if (output->distance > rA + rB && output->distance > kEpsilon) {
            output->distance -= rA + rB;
            Vec2 normal = output->pointB - output->pointA;
            normal.Normalize();
            output->pointA += rA * normal;
            output->pointB -= rB * normal;
        } else {
            Vec2 p = 0.5f * (output->pointA + output->pointB);
            output->pointA = p;
            output->pointB = p;
            output->distance = 0.0f;
        }
    }
}

// collision/b2collision.d:449-467
static bool TestOverlapShapes(const Shape& shapeA, const Shape& shapeB, const Transform& xfA,
                              const Transform& xfB) {
    DistanceInput input;
    input.proxyA.Set(shapeA);
    input.proxyB.Set(shapeB);
    input.transformA = xfA;
    input.transformB = xfB;
    input.useRadii = true;
    SimplexCache cache;
    cache.count = 0;
    DistanceOutput output;
    ComputeDistance(&output, &cache, &input);
    return output.distance < 10.0f * kEpsilon;
}

// ------------------------------------------------------------ time of impact
// collision/b2timeofimpact.d
enum { kToiUnknown = 0, kToiFailed, kToiOverlapped, kToiTouching, kToiSeparated };
struct TOIInput { DistanceProxy proxyA, proxyB; Sweep sweepA, sweepB; f32 tMax = 0; };
struct TOIOutput { int state = kToiUnknown; f32 t = 0; };

enum { kSepPoints = 0, kSepFaceA, kSepFaceB };

struct SeparationFunction {                                             // b2timeofimpact.d:309-528
    const DistanceProxy* proxyA = nullptr;
    const DistanceProxy* proxyB = nullptr;
    Sweep sweepA, sweepB;
    int type = kSepPoints;
    Vec2 localPoint;
    Vec2 axis;
    f32 Initialize(const SimplexCache* cache, const DistanceProxy* pA, const Sweep& sA,
                   const DistanceProxy* pB, const Sweep& sB, f32 t1) {
        proxyA = pA;
        proxyB = pB;
        int count = cache->count;
        sweepA = sA;
        sweepB = sB;
        Transform xfA, xfB;
        sweepA.GetTransform(&xfA, t1);
        sweepB.GetTransform(&xfB, t1);
        if (count == 1) {
            type = kSepPoints;
            Vec2 localPointA = proxyA->GetVertex(cache->indexA[0]);
            Vec2 localPointB = proxyB->GetVertex(cache->indexB[0]);
            Vec2 pointA = Mul(xfA, localPointA);
            Vec2 pointB = Mul(xfB, localPointB);
            axis = pointB - pointA;
            f32 s = axis.Normalize();
            return s;
        } else if (cache->indexA[0] == cache->indexA[1]) {
            type = kSepFaceB;
            Vec2 localPointB1 = pB->GetVertex(cache->indexB[0]);
            Vec2 localPointB2 = pB->GetVertex(cache->indexB[1]);
            axis = Cross(localPointB2 - localPointB1, 1.0f);
            axis.Normalize();
            Vec2 normal = Mul(xfB.q, axis);
            localPoint = 0.5f * (localPointB1 + localPointB2);
            Vec2 pointB = Mul(xfB, localPoint);
            Vec2 localPointA = pA->GetVertex(cache->indexA[0]);
            Vec2 pointA = Mul(xfA, localPointA);
            f32 s = Dot(pointA - pointB, normal);
            if (s < 0.0f) { axis = -axis; s = -s; }
            return s;
        } else {
            type = kSepFaceA;
            Vec2 localPointA1 = proxyA->GetVertex(cache->indexA[0]);
            Vec2 localPointA2 = proxyA->GetVertex(cache->indexA[1]);
            axis = Cross(localPointA2 - localPointA1, 1.0f);
            axis.Normalize();
            Vec2 normal = Mul(xfA.q, axis);
            localPoint = 0.5f * (localPointA1 + localPointA2);
            Vec2 pointA = Mul(xfA, localPoint);
            Vec2 localPointB = proxyB->GetVertex(cache->indexB[0]);
            Vec2 pointB = Mul(xfB, localPointB);
            f32 s = Dot(pointB - pointA, normal);
            if (s < 0.0f) { axis = -axis; s = -s; }
            return s;
        }
    }
    f32 FindMinSeparation(int* indexA, int* indexB, f32 t) const {
        Transform xfA, xfB;
        sweepA.GetTransform(&xfA, t);
        sweepB.GetTransform(&xfB, t);
        switch (type) {
        case kSepPoints: {
            Vec2 axisA = MulT(xfA.q, axis);
            Vec2 axisB = MulT(xfB.q, -axis);
            *indexA = proxyA->GetSupport(axisA);
            *indexB = proxyB->GetSupport(axisB);
            Vec2 localPointA = proxyA->GetVertex(*indexA);
            Vec2 localPointB = proxyB->GetVertex(*indexB);
            Vec2 pointA = Mul(xfA, localPointA);
            Vec2 pointB = Mul(xfB, localPointB);
            return Dot(pointB - pointA, axis);
        }
        case kSepFaceA: {
            Vec2 normal = Mul(xfA.q, axis);
            Vec2 pointA = Mul(xfA, localPoint);
            Vec2 axisB = MulT(xfB.q, -normal);
            *indexA = -1;
            *indexB = proxyB->GetSupport(axisB);
            Vec2 localPointB = proxyB->GetVertex(*indexB);
            Vec2 pointB = Mul(xfB, localPointB);
            return Dot(pointB - pointA, normal);
        }
        default: {
            Vec2 normal = Mul(xfB.q, axis);
            Vec2 pointB = Mul(xfB, localPoint);
            Vec2 axisA = MulT(xfA.q, -normal);
            *indexB = -1;
            *indexA = proxyA->GetSupport(axisA);
            Vec2 localPointA = proxyA->GetVertex(*indexA);
            Vec2 pointA = Mul(xfA, localPointA);
            return Dot(pointA - pointB, normal);
        }
        }
    }
    f32 Evaluate(int indexA, int indexB, f32 t) const {
        Transform xfA, xfB;
        sweepA.GetTransform(&xfA, t);
        sweepB.GetTransform(&xfB, t);
        switch (type) {
        case kSepPoints: {
            Vec2 localPointA = proxyA->GetVertex(indexA);
            Vec2 localPointB = proxyB->GetVertex(indexB);
            Vec2 pointA = Mul(xfA, localPointA);
            Vec2 pointB = Mul(xfB, localPointB);
            return Dot(pointB - pointA, axis);
        }
        case kSepFaceA: {
            Vec2 normal = Mul(xfA.q, axis);
            Vec2 pointA = Mul(xfA, localPoint);
            Vec2 localPointB = proxyB->GetVertex(indexB);
            Vec2 pointB = Mul(xfB, localPointB);
            return Dot(pointB - pointA, normal);
        }
        default: {
            Vec2 normal = Mul(xfB.q, axis);
            Vec2 pointB = Mul(xfB, localPoint);
            Vec2 localPointA = proxyA->GetVertex(indexA);
            Vec2 pointA = Mul(xfA, localPointA);
            return Dot(pointA - pointB, normal);
        }
        }
    }
};

// collision/b2timeofimpact.d:67-302
static void TimeOfImpact(TOIOutput* output, const TOIInput* input) {
    output->state = kToiUnknown;
    output->t = input->tMax;
    const DistanceProxy* proxyA = &input->proxyA;
    const DistanceProxy* proxyB = &input->proxyB;
    Sweep sweepA = input->sweepA;
    Sweep sweepB = input->sweepB;
    sweepA.Normalize();
    sweepB.Normalize();
    f32 tMax = input->tMax;
    f32 totalRadius = proxyA->radius + proxyB->radius;
    f32 target = Max(kLinearSlop, totalRadius - 3.0f * kLinearSlop);
    f32 tolerance = 0.25f * kLinearSlop;
    f32 t1 = 0.0f;
    const int k_maxIterations = 20;
    int iter = 0;
    SimplexCache cache;
    cache.count = 0;
    DistanceInput distanceInput;
    distanceInput.proxyA = input->proxyA;
    distanceInput.proxyB = input->proxyB;
    distanceInput.useRadii = false;
    for (;;) {
        Transform xfA, xfB;
        sweepA.GetTransform(&xfA, t1);
        sweepB.GetTransform(&xfB, t1);
        distanceInput.transformA = xfA;
        distanceInput.transformB = xfB;
        DistanceOutput distanceOutput;
        ComputeDistance(&distanceOutput, &cache, &distanceInput);
        if (distanceOutput.distance <= 0.0f) {
            output->state = kToiOverlapped;
            output->t = 0.0f;
            break;
        }
        if (distanceOutput.distance < target + tolerance) {
            output->state = kToiTouching;
            output->t = t1;
            break;
        }
        SeparationFunction fcn;
        fcn.Initialize(&cache, proxyA, sweepA, proxyB, sweepB, t1);
        bool done = false;
        f32 t2 = tMax;
        int pushBackIter = 0;
        for (;;) {
            int indexA, indexB;
            f32 s2 = fcn.FindMinSeparation(&indexA, &indexB, t2);
            if (s2 > target + tolerance) {
                output->state = kToiSeparated;
                output->t = tMax;
                done = true;
                break;
            }
            if (s2 > target - tolerance) {
                t1 = t2;
                break;
            }
            f32 s1 = fcn.Evaluate(indexA, indexB, t1);
            if (s1 < target - tolerance) {
                output->state = kToiFailed;
                output->t = t1;
                done = true;
                break;
            }
            if (s1 <= target + tolerance) {
                output->state = kToiTouching;
                output->t = t1;
                done = true;
                break;
            }
            int rootIterCount = 0;
            f32 a1 = t1, a2 = t2;
            for (;;) {
                f32 t = 0;
                if (rootIterCount & 1) {
                    t = a1 + ((target - s1) * (a2 - a1)) / (s2 - s1);
                } else {
                    t = 0.5f * (a1 + a2);
                }
                ++rootIterCount;
                f32 s = fcn.Evaluate(indexA, indexB, t);
                if (Abs(s - target) < tolerance) {
                    t2 = t;
                    break;
                }
                if (s > target) { a1 = t; s1 = s; }
                else { a2 = t; s2 = s; }
                if (rootIterCount == 50) break;
            }
            ++pushBackIter;
            if (pushBackIter == kMaxPolygonVertices) break;
        }
        ++iter;
        if (done) break;
        if (iter == k_maxIterations) {
            output->state = kToiFailed;
            output->t = t1;
            break;
        }
    }
}

// ------------------------------------------------------------ dynamic tree
// collision/b2dynamictree.d
static const int kNullNode = -1;
struct TreeNode {
    AABB aabb;
    void* userData = nullptr;
    int parent = kNullNode;   // also "next" for the free list (union in the reference)
    int child1 = kNullNode;
    int child2 = kNullNode;
    int height = 0;
    bool IsLeaf() const { return child1 == kNullNode; }
};

struct DynamicTree {
    int root = kNullNode;
    std::vector<TreeNode> nodes;
    int nodeCount = 0;
    int freeList = 0;

    DynamicTree() {                                                     // b2dynamictree.d:82-107
        nodes.resize(16);
        for (int i = 0; i < 16 - 1; ++i) { nodes[i].parent = i + 1; nodes[i].height = -1; }
        nodes[15].parent = kNullNode;
        nodes[15].height = -1;
        freeList = 0;
    }
    int AllocateNode() {                                                // b2dynamictree.d:516-551
        if (freeList == kNullNode) {
            int oldCap = (int)nodes.size();
            int cap = oldCap * 2;
            nodes.resize(cap);
            for (int i = nodeCount; i < cap - 1; ++i) { nodes[i].parent = i + 1; nodes[i].height = -1; }
            nodes[cap - 1].parent = kNullNode;
            nodes[cap - 1].height = -1;
            freeList = nodeCount;
        }
        int nodeId = freeList;
        freeList = nodes[nodeId].parent;
        nodes[nodeId].parent = kNullNode;
        nodes[nodeId].child1 = kNullNode;
        nodes[nodeId].child2 = kNullNode;
        nodes[nodeId].height = 0;
        nodes[nodeId].userData = nullptr;
        ++nodeCount;
        return nodeId;
    }
    void FreeNode(int nodeId) {                                         // b2dynamictree.d:554-564
        nodes[nodeId].parent = freeList;
        nodes[nodeId].height = -1;
        freeList = nodeId;
        --nodeCount;
    }
    int CreateProxy(const AABB& aabb, void* userData) {                 // b2dynamictree.d:110-124
        int proxyId = AllocateNode();
        Vec2 r(kAabbExtension, kAabbExtension);
        nodes[proxyId].aabb.lowerBound = aabb.lowerBound - r;
        nodes[proxyId].aabb.upperBound = aabb.upperBound + r;
        nodes[proxyId].userData = userData;
        nodes[proxyId].height = 0;
        InsertLeaf(proxyId);
        return proxyId;
    }
    void DestroyProxy(int proxyId) {                                    // b2dynamictree.d:127-134
        RemoveLeaf(proxyId);
        FreeNode(proxyId);
    }
    bool MoveProxy(int proxyId, const AABB& aabb, Vec2 displacement) {  // b2dynamictree.d:140-184
        if (nodes[proxyId].aabb.Contains(aabb)) return false;
        RemoveLeaf(proxyId);
        AABB b = aabb;
        Vec2 r(kAabbExtension, kAabbExtension);
        b.lowerBound = b.lowerBound - r;
        b.upperBound = b.upperBound + r;
        Vec2 d = kAabbMultiplier * displacement;
        if (d.x < 0.0f) b.lowerBound.x += d.x; else b.upperBound.x += d.x;
        if (d.y < 0.0f) b.lowerBound.y += d.y; else b.upperBound.y += d.y;
        nodes[proxyId].aabb = b;
        InsertLeaf(proxyId);
        return true;
    }
    template <class CB> void Query(CB* callback, const AABB& aabb) const {  // b2dynamictree.d:203-237
        std::vector<int> stack;
        stack.reserve(256);
        stack.push_back(root);
        while (!stack.empty()) {
            int nodeId = stack.back();
            stack.pop_back();
            if (nodeId == kNullNode) continue;
            const TreeNode* node = &nodes[nodeId];
            if (TestOverlap(node->aabb, aabb)) {
                if (node->IsLeaf()) {
                    if (!callback->QueryCallback(nodeId)) return;
                } else {
                    stack.push_back(node->child1);
                    stack.push_back(node->child2);
                }
            }
        }
    }
    // b2dynamictree.d:246-331: callback->RayCastCallback(p1, p2, maxFraction, proxyId) returns
    // 0 to stop, a positive value to clip the ray to it, a negative one to go on unchanged
    template <class CB> void RayCast(CB* callback, Vec2 p1, Vec2 p2, f32 inputMaxFraction) const {
        Vec2 r = p2 - p1;
        r.Normalize();
        Vec2 v = Cross(1.0f, r);
        Vec2 abs_v(Abs(v.x), Abs(v.y));
        f32 maxFraction = inputMaxFraction;
        AABB segmentAABB;
        {
            Vec2 t = p1 + maxFraction * (p2 - p1);
            segmentAABB.lowerBound = Min(p1, t);
            segmentAABB.upperBound = Max(p1, t);
        }
        std::vector<int> stack;
        stack.reserve(256);
        stack.push_back(root);
        while (!stack.empty()) {
            int nodeId = stack.back();
            stack.pop_back();
            if (nodeId == kNullNode) continue;
            const TreeNode* node = &nodes[nodeId];
            if (!TestOverlap(node->aabb, segmentAABB)) continue;
            Vec2 c = 0.5f * (node->aabb.lowerBound + node->aabb.upperBound);
            Vec2 h = 0.5f * (node->aabb.upperBound - node->aabb.lowerBound);
            f32 separation = Abs(Dot(v, p1 - c)) - Dot(abs_v, h);
            if (separation > 0.0f) continue;
            if (node->IsLeaf()) {
                f32 value = callback->RayCastCallback(p1, p2, maxFraction, nodeId);
                if (value == 0.0f) return;
                if (value > 0.0f) {
                    maxFraction = value;
                    Vec2 t = p1 + maxFraction * (p2 - p1);
                    segmentAABB.lowerBound = Min(p1, t);
                    segmentAABB.upperBound = Max(p1, t);
                }
            } else {
                stack.push_back(node->child1);
                stack.push_back(node->child2);
            }
        }
    }
    void InsertLeaf(int leaf) {                                         // b2dynamictree.d:566-708
        if (root == kNullNode) {
            root = leaf;
            nodes[root].parent = kNullNode;
            return;
        }
        AABB leafAABB = nodes[leaf].aabb;
        int index = root;
        while (!nodes[index].IsLeaf()) {
            int child1 = nodes[index].child1;
            int child2 = nodes[index].child2;
            f32 area = nodes[index].aabb.GetPerimeter();
            AABB combinedAABB;
            combinedAABB.Combine(nodes[index].aabb, leafAABB);
            f32 combinedArea = combinedAABB.GetPerimeter();
            f32 cost = 2.0f * combinedArea;
            f32 inheritanceCost = 2.0f * (combinedArea - area);
            f32 cost1 = 0;
            if (nodes[child1].IsLeaf()) {
                AABB aabb;
                aabb.Combine(leafAABB, nodes[child1].aabb);
                cost1 = aabb.GetPerimeter() + inheritanceCost;
            } else {
                AABB aabb;
                aabb.Combine(leafAABB, nodes[child1].aabb);
                f32 oldArea = nodes[child1].aabb.GetPerimeter();
                f32 newArea = aabb.GetPerimeter();
                cost1 = (newArea - oldArea) + inheritanceCost;
            }
            f32 cost2 = 0;
            if (nodes[child2].IsLeaf()) {
                AABB aabb;
                aabb.Combine(leafAABB, nodes[child2].aabb);
                cost2 = aabb.GetPerimeter() + inheritanceCost;
            } else {
                AABB aabb;
                aabb.Combine(leafAABB, nodes[child2].aabb);
                f32 oldArea = nodes[child2].aabb.GetPerimeter();
                f32 newArea = aabb.GetPerimeter();
                cost2 = (newArea - oldArea) + inheritanceCost;
            }
            if (cost < cost1 && cost < cost2) break;
            if (cost1 < cost2) index = child1; else index = child2;
        }
        int sibling = index;
        int oldParent = nodes[sibling].parent;
        int newParent = AllocateNode();
        nodes[newParent].parent = oldParent;
        nodes[newParent].userData = nullptr;
        nodes[newParent].aabb.Combine(leafAABB, nodes[sibling].aabb);
        nodes[newParent].height = nodes[sibling].height + 1;
        if (oldParent != kNullNode) {
            if (nodes[oldParent].child1 == sibling) nodes[oldParent].child1 = newParent;
            else nodes[oldParent].child2 = newParent;
            nodes[newParent].child1 = sibling;
            nodes[newParent].child2 = leaf;
            nodes[sibling].parent = newParent;
            nodes[leaf].parent = newParent;
        } else {
            nodes[newParent].child1 = sibling;
            nodes[newParent].child2 = leaf;
            nodes[sibling].parent = newParent;
            nodes[leaf].parent = newParent;
            root = newParent;
        }
        index = nodes[leaf].parent;
        while (index != kNullNode) {
            index = Balance(index);
            int child1 = nodes[index].child1;
            int child2 = nodes[index].child2;
            nodes[index].height = 1 + Max(nodes[child1].height, nodes[child2].height);
            nodes[index].aabb.Combine(nodes[child1].aabb, nodes[child2].aabb);
            index = nodes[index].parent;
        }
    }
    void RemoveLeaf(int leaf) {                                         // b2dynamictree.d:710-769
        if (leaf == root) { root = kNullNode; return; }
        int parent = nodes[leaf].parent;
        int grandParent = nodes[parent].parent;
        int sibling = nodes[parent].child1 == leaf ? nodes[parent].child2 : nodes[parent].child1;
        if (grandParent != kNullNode) {
            if (nodes[grandParent].child1 == parent) nodes[grandParent].child1 = sibling;
            else nodes[grandParent].child2 = sibling;
            nodes[sibling].parent = grandParent;
            FreeNode(parent);
            int index = grandParent;
            while (index != kNullNode) {
                index = Balance(index);
                int child1 = nodes[index].child1;
                int child2 = nodes[index].child2;
                nodes[index].aabb.Combine(nodes[child1].aabb, nodes[child2].aabb);
                nodes[index].height = 1 + Max(nodes[child1].height, nodes[child2].height);
                index = nodes[index].parent;
            }
        } else {
            root = sibling;
            nodes[sibling].parent = kNullNode;
            FreeNode(parent);
        }
    }
    int Balance(int iA) {                                               // b2dynamictree.d:773-915
        TreeNode* A = &nodes[iA];
        if (A->IsLeaf() || A->height < 2) return iA;
        int iB = A->child1;
        int iC = A->child2;
        TreeNode* B = &nodes[iB];
        TreeNode* C = &nodes[iC];
        int balance = C->height - B->height;
        if (balance > 1) {
            int iF = C->child1;
            int iG = C->child2;
            TreeNode* F = &nodes[iF];
            TreeNode* G = &nodes[iG];
            C->child1 = iA;
            C->parent = A->parent;
            A->parent = iC;
            if (C->parent != kNullNode) {
                if (nodes[C->parent].child1 == iA) nodes[C->parent].child1 = iC;
                else nodes[C->parent].child2 = iC;
            } else {
                root = iC;
            }
            if (F->height > G->height) {
                C->child2 = iF;
                A->child2 = iG;
                G->parent = iA;
                A->aabb.Combine(B->aabb, G->aabb);
                C->aabb.Combine(A->aabb, F->aabb);
                A->height = 1 + Max(B->height, G->height);
                C->height = 1 + Max(A->height, F->height);
            } else {
                C->child2 = iG;
                A->child2 = iF;
                F->parent = iA;
                A->aabb.Combine(B->aabb, F->aabb);
                C->aabb.Combine(A->aabb, G->aabb);
                A->height = 1 + Max(B->height, F->height);
                C->height = 1 + Max(A->height, G->height);
            }
            return iC;
        }
        if (balance < -1) {
            int iD = B->child1;
            int iE = B->child2;
            TreeNode* D = &nodes[iD];
            TreeNode* E = &nodes[iE];
            B->child1 = iA;
            B->parent = A->parent;
            A->parent = iB;
            if (B->parent != kNullNode) {
                if (nodes[B->parent].child1 == iA) nodes[B->parent].child1 = iB;
                else nodes[B->parent].child2 = iB;
            } else {
                root = iB;
            }
            if (D->height > E->height) {
                B->child2 = iD;
                A->child1 = iE;
                E->parent = iA;
                A->aabb.Combine(C->aabb, E->aabb);
                B->aabb.Combine(A->aabb, D->aabb);
                A->height = 1 + Max(C->height, E->height);
                B->height = 1 + Max(A->height, D->height);
            } else {
                B->child2 = iE;
                A->child1 = iD;
                D->parent = iA;
                A->aabb.Combine(C->aabb, D->aabb);
                B->aabb.Combine(A->aabb, E->aabb);
                A->height = 1 + Max(C->height, D->height);
                B->height = 1 + Max(A->height, E->height);
            }
            return iB;
        }
        return iA;
    }
};

// ------------------------------------------------------------ world objects
struct Body;
struct Fixture;
struct Contact;
struct Joint;
struct World;

struct ContactEdge { Body* other = nullptr; Contact* contact = nullptr; ContactEdge* prev = nullptr; ContactEdge* next = nullptr; };
struct JointEdge { Body* other = nullptr; Joint* joint = nullptr; JointEdge* prev = nullptr; JointEdge* next = nullptr; };

struct FixtureProxy { AABB aabb; Fixture* fixture = nullptr; int childIndex = 0; int proxyId = -1; };

struct Filter { uint16_t categoryBits = 0x0001; uint16_t maskBits = 0xFFFF; int16_t groupIndex = 0; };

struct Fixture {                                                        // dynamics/b2fixture.d
    f32 density = 0;
    Fixture* next = nullptr;
    Body* body = nullptr;
    Shape shape;
    f32 friction = 0;
    f32 restitution = 0;
    FixtureProxy proxy;
    int proxyCount = 0;
    Filter filter;
    bool isSensor = false;
    int index = 0;   // creation order (for export)
    int chain = -1;  // the b2ChainShape this child edge belongs to (World::chains), or -1
    int fclass = 0;  // user data a table contact filter reads (stands in for b2Fixture.m_userData)
};

enum { kStaticBody = 0, kKinematicBody = 1, kDynamicBody = 2 };
enum {                                                                  // b2body.d:1118-1127
    kBodyIsland = 0x0001, kBodyAwake = 0x0002, kBodyAutoSleep = 0x0004, kBodyBullet = 0x0008,
    kBodyFixedRotation = 0x0010, kBodyActive = 0x0020, kBodyToi = 0x0040
};

struct Body {
    int type = kStaticBody;
    uint16_t flags = 0;
    int islandIndex = 0;
    Transform xf;
    Sweep sweep;
    Vec2 linearVelocity;
    f32 angularVelocity = 0;
    Vec2 force;
    f32 torque = 0;
    World* world = nullptr;
    Body* prev = nullptr;
    Body* next = nullptr;
    Fixture* fixtureList = nullptr;
    int fixtureCount = 0;
    JointEdge* jointList = nullptr;
    ContactEdge* contactList = nullptr;
    f32 mass = 0, invMass = 0;
    f32 I = 0, invI = 0;
    f32 linearDamping = 0, angularDamping = 0, gravityScale = 0;
    f32 sleepTime = 0;
    int index = 0;

    bool IsAwake() const { return (flags & kBodyAwake) == kBodyAwake; }
    bool IsActive() const { return (flags & kBodyActive) == kBodyActive; }
    bool IsBullet() const { return (flags & kBodyBullet) == kBodyBullet; }
    void SetAwake(bool flag) {                                          // b2body.d:827-846
        if (flag) {
            if ((flags & kBodyAwake) == 0) { flags |= kBodyAwake; sleepTime = 0.0f; }
        } else {
            flags &= ~kBodyAwake;
            sleepTime = 0.0f;
            linearVelocity.SetZero();
            angularVelocity = 0.0f;
            force.SetZero();
            torque = 0.0f;
        }
    }
    void SynchronizeTransform() {                                       // b2body.d:1143-1147
        xf.q.Set(sweep.a);
        xf.p = sweep.c - Mul(xf.q, sweep.localCenter);
    }
    void Advance(f32 alpha) {                                           // b2body.d:1172-1180
        sweep.Advance(alpha);
        sweep.c = sweep.c0;
        sweep.a = sweep.a0;
        xf.q.Set(sweep.a);
        xf.p = sweep.c - Mul(xf.q, sweep.localCenter);
    }
    bool ShouldCollide(const Body* other) const;
    void SynchronizeFixtures();
    void ResetMassData();
};

enum {                                                                  // b2contact.d:242-261
    kContactIsland = 0x0001, kContactTouching = 0x0002, kContactEnabled = 0x0004,
    kContactFilter = 0x0008, kContactBulletHit = 0x0010, kContactToi = 0x0020
};

struct Listener;

struct Contact {
    uint32_t flags = 0;
    Contact* prev = nullptr;
    Contact* next = nullptr;
    ContactEdge nodeA, nodeB;
    Fixture* fixtureA = nullptr;
    Fixture* fixtureB = nullptr;
    int indexA = 0, indexB = 0;
    Manifold manifold;
    int toiCount = 0;
    f32 toi = 0;
    f32 friction = 0, restitution = 0, tangentSpeed = 0;

    bool IsTouching() const { return (flags & kContactTouching) == kContactTouching; }
    bool IsEnabled() const { return (flags & kContactEnabled) == kContactEnabled; }
    void SetEnabled(bool f) { if (f) flags |= kContactEnabled; else flags &= ~kContactEnabled; }
    void Evaluate(Manifold* m, const Transform& xfA, const Transform& xfB) {
        const Shape& a = fixtureA->shape;
        const Shape& b = fixtureB->shape;
        if (a.type == kPolygon && b.type == kPolygon) CollidePolygons(m, a, xfA, b, xfB);
        else if (a.type == kPolygon && b.type == kCircle) CollidePolygonAndCircle(m, a, xfA, b, xfB);
        else if (a.type == kEdge && b.type == kCircle) CollideEdgeAndCircle(m, a, xfA, b, xfB);
        else if (a.type == kEdge && b.type == kPolygon) CollideEdgeAndPolygon(m, a, xfA, b, xfB);
        else CollideCircles(m, a, xfA, b, xfB);
    }
    void Update(Listener* listener);
};

// Recording listener: stands in for a user b2ContactListener (b2worldcallbacks.d:87-128).
struct Listener {
    std::vector<dbox_contact_event> events;
    bool record = false;                 // keep the events
    dbox_presolve_fn presolve = nullptr; // a user's PreSolve, called with one record per call
    void* presolve_user = nullptr;
    bool inToi = false;                  // calls made by SolveTOI's sub-step updates
    void Push(int kind, const Contact* c, int pointCount, const f32* ni, const f32* ti) {
        if (!record) return;
        dbox_contact_event e;
        memset(&e, 0, sizeof(e));
        e.kind = kind;
        e.fixture_a = c->fixtureA->index;
        e.fixture_b = c->fixtureB->index;
        e.point_count = pointCount;
        for (int i = 0; i < pointCount && i < 2; ++i) {
            e.normal_impulses[i] = ni ? ni[i] : 0.0f;
            e.tangent_impulses[i] = ti ? ti[i] : 0.0f;
        }
        events.push_back(e);
    }
    void BeginContact(Contact* c) { Push(DBOX_EVENT_BEGIN, c, c->manifold.pointCount, nullptr, nullptr); }
    void EndContact(Contact* c) { Push(DBOX_EVENT_END, c, c->manifold.pointCount, nullptr, nullptr); }
    void PreSolve(Contact* c, const Manifold*);
    void PostSolve(Contact* c, int count, const f32* ni, const f32* ti) { Push(DBOX_EVENT_POSTSOLVE, c, count, ni, ti); }
};

void FillContactState(const Contact* c, dbox_contact_state* o) {
    memset(o, 0, sizeof(*o));
    o->fixture_a = c->fixtureA->index;
    o->fixture_b = c->fixtureB->index;
    o->flags = c->flags;
    o->toi_count = c->toiCount;
    o->toi = c->toi;
    o->friction = c->friction;
    o->restitution = c->restitution;
    o->tangent_speed = c->tangentSpeed;
    o->point_count = c->manifold.pointCount;
    o->type = c->manifold.type;
    o->local_normal[0] = c->manifold.localNormal.x; o->local_normal[1] = c->manifold.localNormal.y;
    o->local_point[0] = c->manifold.localPoint.x; o->local_point[1] = c->manifold.localPoint.y;
    for (int k = 0; k < c->manifold.pointCount; ++k) {
        const ManifoldPoint& mp = c->manifold.points[k];
        o->points[k].local_point[0] = mp.localPoint.x;
        o->points[k].local_point[1] = mp.localPoint.y;
        o->points[k].normal_impulse = mp.normalImpulse;
        o->points[k].tangent_impulse = mp.tangentImpulse;
        o->points[k].id = mp.id.key;
    }
}


// b2ContactListener.PreSolve (b2worldcallbacks.d:101-115): the user's callback may call
// SetEnabled / SetFriction / SetRestitution / SetTangentSpeed (contacts/b2contact.d:105-190)
void Listener::PreSolve(Contact* c, const Manifold*) {
    Push(DBOX_EVENT_PRESOLVE, c, c->manifold.pointCount, nullptr, nullptr);
    if (!presolve) return;
    dbox_presolve_contact r;
    memset(&r, 0, sizeof(r));
    r.world = inToi ? -1 : 0;            // test aid: -1 marks a call from SolveTOI
    r.enabled = c->IsEnabled() ? 1 : 0;
    r.friction = c->friction;
    r.restitution = c->restitution;
    r.tangent_speed = c->tangentSpeed;
    FillContactState(c, &r.contact);
    presolve(&r, 1, presolve_user);
    c->SetEnabled(r.enabled != 0);
    c->friction = r.friction;
    c->restitution = r.restitution;
    c->tangentSpeed = r.tangent_speed;
}

// b2contact.d:32-42
static inline f32 MixFriction(f32 f1, f32 f2) { return sqrtf(f1 * f2); }
static inline f32 MixRestitution(f32 r1, f32 r2) { return r1 > r2 ? r1 : r2; }

// contacts/b2contact.d:270-356
void Contact::Update(Listener* listener) {
    Manifold oldManifold = manifold;
    flags |= kContactEnabled;
    bool touching = false;
    bool wasTouching = (flags & kContactTouching) == kContactTouching;
    bool sensorA = fixtureA->isSensor;
    bool sensorB = fixtureB->isSensor;
    bool sensor = sensorA || sensorB;
    Body* bodyA = fixtureA->body;
    Body* bodyB = fixtureB->body;
    Transform xfA = bodyA->xf;
    Transform xfB = bodyB->xf;
    if (sensor) {
        touching = TestOverlapShapes(fixtureA->shape, fixtureB->shape, xfA, xfB);
        manifold.pointCount = 0;
    } else {
        Evaluate(&manifold, xfA, xfB);
        touching = manifold.pointCount > 0;
        for (int i = 0; i < manifold.pointCount; ++i) {
            ManifoldPoint* mp2 = manifold.points + i;
            mp2->normalImpulse = 0.0f;
            mp2->tangentImpulse = 0.0f;
            ContactID id2 = mp2->id;
            for (int j = 0; j < oldManifold.pointCount; ++j) {
                ManifoldPoint* mp1 = oldManifold.points + j;
                if (mp1->id.key == id2.key) {
                    mp2->normalImpulse = mp1->normalImpulse;
                    mp2->tangentImpulse = mp1->tangentImpulse;
                    break;
                }
            }
        }
        if (touching != wasTouching) {
            bodyA->SetAwake(true);
            bodyB->SetAwake(true);
        }
    }
    if (touching) flags |= kContactTouching; else flags &= ~kContactTouching;
    if (!wasTouching && touching && listener) listener->BeginContact(this);
    if (wasTouching && !touching && listener) listener->EndContact(this);
    if (!sensor && touching && listener) listener->PreSolve(this, &oldManifold);
}

// ------------------------------------------------------------ revolute joint
enum { kInactiveLimit = 0, kAtLowerLimit, kAtUpperLimit, kEqualLimits };

struct Position { Vec2 c; f32 a = 0; };
struct Velocity { Vec2 v; f32 w = 0; };
struct TimeStep { f32 dt = 0, inv_dt = 0, dtRatio = 0; int velocityIterations = 0, positionIterations = 0; bool warmStarting = false; };
struct SolverData { TimeStep step; Position* positions = nullptr; Velocity* velocities = nullptr; };

enum { kRevoluteJoint = 0, kDistanceJoint = 1, kRopeJoint = 2, kWeldJoint = 3, kFrictionJoint = 4, kMotorJoint = 5,
       kWheelJoint = 6, kPrismaticJoint = 7, kPulleyJoint = 8, kMouseJoint = 9, kGearJoint = 10 };

struct Joint {                                                          // joints/b2joint.d, b2revolutejoint.d, b2distancejoint.d
    int type = kRevoluteJoint;
    Joint* prev = nullptr;
    Joint* next = nullptr;
    JointEdge edgeA, edgeB;
    Body* bodyA = nullptr;
    Body* bodyB = nullptr;
    bool islandFlag = false;
    bool collideConnected = false;
    int index = 0;
    // revolute
    Vec2 localAnchorA, localAnchorB;
    Vec3 impulse;
    f32 motorImpulse = 0;
    bool enableMotor = false;
    f32 maxMotorTorque = 0, motorSpeed = 0;
    bool enableLimit = false;
    f32 referenceAngle = 0, lowerAngle = 0, upperAngle = 0;
    int indexA = 0, indexB = 0;
    Vec2 rA, rB, localCenterA, localCenterB;
    f32 invMassA = 0, invMassB = 0, invIA = 0, invIB = 0;
    Mat33 massM;
    f32 motorMass = 0;
    int limitState = kInactiveLimit;
    // distance and rope (the impulse is impulse.x; the rope's maximum length is `length`,
    // its state limitState); weld (referenceAngle, frequency, damping, gamma, bias; its
    // mass matrix is massM)
    f32 length = 0, frequencyHz = 0, dampingRatio = 0, gamma = 0, bias = 0, distMass = 0;
    f32 curLength = 0;
    Vec2 u;
    // friction and motor (linear impulse impulse.x/.y, angular impulse impulse.z)
    f32 maxForce = 0, maxTorque = 0, correctionFactor = 0, angularOffset = 0, angularError = 0, angularMass = 0;
    Vec2 linearOffset, linearError;
    Mat22 linearMass;
    // wheel (point-to-line impulse impulse.x, spring impulse impulse.y, motorImpulse)
    Vec2 localXAxisA, localYAxisA, ax, ay;
    f32 sAx = 0, sBx = 0, sAy = 0, sBy = 0, wheelMass = 0, springMass = 0;
    // prismatic (impulse: perpendicular, angular, limit; K in massM)
    f32 lowerTranslation = 0, upperTranslation = 0, maxMotorForce = 0;
    Vec2 axis, perp;
    f32 s1 = 0, s2 = 0, a1 = 0, a2 = 0;
    // pulley (impulse.x) and mouse (impulse.x/.y; mass matrix in linearMass)
    Vec2 groundAnchorA, groundAnchorB, uA, uB, targetA, mouseC;
    f32 ratio = 0, constant = 0, beta = 0, lengthA = 0, lengthB = 0;
    int dumpIndex = 0;           // b2Joint.m_index: the joint's place in the world list, set by Dump
    // gear (b2gearjoint.d): joint1 joins bodyC (its A) to bodyA (its B), joint2 bodyD to bodyB;
    // the impulse is impulse.x, the ratio and constant the pulley's fields
    Joint* joint1 = nullptr;
    Joint* joint2 = nullptr;
    int typeA = 0, typeB = 0;
    Body* bodyC = nullptr;
    Body* bodyD = nullptr;
    int indexC = 0, indexD = 0;
    Vec2 localAnchorC, localAnchorD, localAxisC, localAxisD, lcC, lcD, JvAC, JvBD;
    f32 referenceAngleA = 0, referenceAngleB = 0, JwA = 0, JwB = 0, JwC = 0, JwD = 0, mC = 0, mD = 0, iC = 0, iD = 0;
    f32 gearMass = 0;

    void InitVelocityConstraints(const SolverData& data) {
        switch (type) {
        case kDistanceJoint: DistanceInit(data); break;
        case kRopeJoint: RopeInit(data); break;
        case kWeldJoint: WeldInit(data); break;
        case kFrictionJoint:
        case kMotorJoint: FrictionMotorInit(data); break;
        case kWheelJoint: WheelInit(data); break;
        case kPrismaticJoint: PrismaticInit(data); break;
        case kPulleyJoint: PulleyInit(data); break;
        case kMouseJoint: MouseInit(data); break;
        case kGearJoint: GearInit(data); break;
        default: RevoluteInit(data);
        }
    }
    void SolveVelocityConstraints(const SolverData& data) {
        switch (type) {
        case kDistanceJoint: DistanceSolveVelocity(data); break;
        case kRopeJoint: RopeSolveVelocity(data); break;
        case kWeldJoint: WeldSolveVelocity(data); break;
        case kFrictionJoint:
        case kMotorJoint: FrictionMotorSolveVelocity(data); break;
        case kWheelJoint: WheelSolveVelocity(data); break;
        case kPrismaticJoint: PrismaticSolveVelocity(data); break;
        case kPulleyJoint: PulleySolveVelocity(data); break;
        case kMouseJoint: MouseSolveVelocity(data); break;
        case kGearJoint: GearSolveVelocity(data); break;
        default: RevoluteSolveVelocity(data);
        }
    }
    bool SolvePositionConstraints(const SolverData& data) {
        switch (type) {
        case kDistanceJoint: return DistanceSolvePosition(data);
        case kRopeJoint: return RopeSolvePosition(data);
        case kWeldJoint: return WeldSolvePosition(data);
        case kFrictionJoint:
        case kMotorJoint: return true;                                 // no position correction
        case kWheelJoint: return WheelSolvePosition(data);
        case kPrismaticJoint: return PrismaticSolvePosition(data);
        case kPulleyJoint: return PulleySolvePosition(data);
        case kMouseJoint: return true;
        case kGearJoint: return GearSolvePosition(data);
        default: return RevoluteSolvePosition(data);
        }
    }

    void LoadBodies() {
        indexA = bodyA->islandIndex;
        indexB = bodyB->islandIndex;
        localCenterA = bodyA->sweep.localCenter;
        localCenterB = bodyB->sweep.localCenter;
        invMassA = bodyA->invMass;
        invMassB = bodyB->invMass;
        invIA = bodyA->invI;
        invIB = bodyB->invI;
    }

    void GearInit(const SolverData& data) {                             // b2gearjoint.d:245-350
        LoadBodies();
        indexC = bodyC->islandIndex;
        indexD = bodyD->islandIndex;
        lcC = bodyC->sweep.localCenter;
        lcD = bodyD->sweep.localCenter;
        mC = bodyC->invMass;
        mD = bodyD->invMass;
        iC = bodyC->invI;
        iD = bodyD->invI;
        f32 aA = data.positions[indexA].a, aB = data.positions[indexB].a;
        f32 aC = data.positions[indexC].a, aD = data.positions[indexD].a;
        Vec2 vA = data.velocities[indexA].v, vB = data.velocities[indexB].v;
        Vec2 vC = data.velocities[indexC].v, vD = data.velocities[indexD].v;
        f32 wA = data.velocities[indexA].w, wB = data.velocities[indexB].w;
        f32 wC = data.velocities[indexC].w, wD = data.velocities[indexD].w;
        Rot qA(aA), qB(aB), qC(aC), qD(aD);
        gearMass = 0.0f;
        if (typeA == kRevoluteJoint) {
            JvAC.SetZero();
            JwA = 1.0f;
            JwC = 1.0f;
            gearMass += invIA + iC;
        } else {
            Vec2 u = Mul(qC, localAxisC);
            Vec2 rC = Mul(qC, localAnchorC - lcC);
            Vec2 rA2 = Mul(qA, localAnchorA - localCenterA);
            JvAC = u;
            JwC = Cross(rC, u);
            JwA = Cross(rA2, u);
            gearMass += mC + invMassA + iC * JwC * JwC + invIA * JwA * JwA;
        }
        if (typeB == kRevoluteJoint) {
            JvBD.SetZero();
            JwB = ratio;
            JwD = ratio;
            gearMass += ratio * ratio * (invIB + iD);
        } else {
            Vec2 u = Mul(qD, localAxisD);
            Vec2 rD = Mul(qD, localAnchorD - lcD);
            Vec2 rB2 = Mul(qB, localAnchorB - localCenterB);
            JvBD = ratio * u;
            JwD = ratio * Cross(rD, u);
            JwB = ratio * Cross(rB2, u);
            gearMass += ratio * ratio * (mD + invMassB) + iD * JwD * JwD + invIB * JwB * JwB;
        }
        gearMass = gearMass > 0.0f ? 1.0f / gearMass : 0.0f;
        if (data.step.warmStarting) {
            vA += (invMassA * impulse.x) * JvAC;
            wA += invIA * impulse.x * JwA;
            vB += (invMassB * impulse.x) * JvBD;
            wB += invIB * impulse.x * JwB;
            vC -= (mC * impulse.x) * JvAC;
            wC -= iC * impulse.x * JwC;
            vD -= (mD * impulse.x) * JvBD;
            wD -= iD * impulse.x * JwD;
        } else {
            impulse.x = 0.0f;
        }
        data.velocities[indexA].v = vA;
        data.velocities[indexA].w = wA;
        data.velocities[indexB].v = vB;
        data.velocities[indexB].w = wB;
        data.velocities[indexC].v = vC;
        data.velocities[indexC].w = wC;
        data.velocities[indexD].v = vD;
        data.velocities[indexD].w = wD;
    }

    void GearSolveVelocity(const SolverData& data) {                    // b2gearjoint.d:352-386
        Vec2 vA = data.velocities[indexA].v, vB = data.velocities[indexB].v;
        Vec2 vC = data.velocities[indexC].v, vD = data.velocities[indexD].v;
        f32 wA = data.velocities[indexA].w, wB = data.velocities[indexB].w;
        f32 wC = data.velocities[indexC].w, wD = data.velocities[indexD].w;
        f32 Cdot = Dot(JvAC, vA - vC) + Dot(JvBD, vB - vD);
        Cdot += (JwA * wA - JwC * wC) + (JwB * wB - JwD * wD);
        f32 imp = -gearMass * Cdot;
        impulse.x += imp;
        vA += (invMassA * imp) * JvAC;
        wA += invIA * imp * JwA;
        vB += (invMassB * imp) * JvBD;
        wB += invIB * imp * JwB;
        vC -= (mC * imp) * JvAC;
        wC -= iC * imp * JwC;
        vD -= (mD * imp) * JvBD;
        wD -= iD * imp * JwD;
        data.velocities[indexA].v = vA;
        data.velocities[indexA].w = wA;
        data.velocities[indexB].v = vB;
        data.velocities[indexB].w = wB;
        data.velocities[indexC].v = vC;
        data.velocities[indexC].w = wC;
        data.velocities[indexD].v = vD;
        data.velocities[indexD].w = wD;
    }

    bool GearSolvePosition(const SolverData& data) {                    // b2gearjoint.d:388-500
        Vec2 cA = data.positions[indexA].c, cB = data.positions[indexB].c;
        Vec2 cC = data.positions[indexC].c, cD = data.positions[indexD].c;
        f32 aA = data.positions[indexA].a, aB = data.positions[indexB].a;
        f32 aC = data.positions[indexC].a, aD = data.positions[indexD].a;
        Rot qA(aA), qB(aB), qC(aC), qD(aD);
        f32 coordinateA = 0, coordinateB = 0;
        Vec2 jvAC, jvBD;
        f32 jwA = 0, jwB = 0, jwC = 0, jwD = 0;
        f32 mass = 0.0f;
        if (typeA == kRevoluteJoint) {
            jvAC.SetZero();
            jwA = 1.0f;
            jwC = 1.0f;
            mass += invIA + iC;
            coordinateA = aA - aC - referenceAngleA;
        } else {
            Vec2 u = Mul(qC, localAxisC);
            Vec2 rC = Mul(qC, localAnchorC - lcC);
            Vec2 rA2 = Mul(qA, localAnchorA - localCenterA);
            jvAC = u;
            jwC = Cross(rC, u);
            jwA = Cross(rA2, u);
            mass += mC + invMassA + iC * jwC * jwC + invIA * jwA * jwA;
            Vec2 pC = localAnchorC - lcC;
            Vec2 pA = MulT(qC, rA2 + (cA - cC));
            coordinateA = Dot(pA - pC, localAxisC);
        }
        if (typeB == kRevoluteJoint) {
            jvBD.SetZero();
            jwB = ratio;
            jwD = ratio;
            mass += ratio * ratio * (invIB + iD);
            coordinateB = aB - aD - referenceAngleB;
        } else {
            Vec2 u = Mul(qD, localAxisD);
            Vec2 rD = Mul(qD, localAnchorD - lcD);
            Vec2 rB2 = Mul(qB, localAnchorB - localCenterB);
            jvBD = ratio * u;
            jwD = ratio * Cross(rD, u);
            jwB = ratio * Cross(rB2, u);
            mass += ratio * ratio * (mD + invMassB) + iD * jwD * jwD + invIB * jwB * jwB;
            Vec2 pD = localAnchorD - lcD;
            Vec2 pB = MulT(qD, rB2 + (cB - cD));
            coordinateB = Dot(pB - pD, localAxisD);
        }
        f32 C = (coordinateA + ratio * coordinateB) - constant;
        f32 imp = 0.0f;
        if (mass > 0.0f) imp = -C / mass;
        cA += invMassA * imp * jvAC;
        aA += invIA * imp * jwA;
        cB += invMassB * imp * jvBD;
        aB += invIB * imp * jwB;
        cC -= mC * imp * jvAC;
        aC -= iC * imp * jwC;
        cD -= mD * imp * jvBD;
        aD -= iD * imp * jwD;
        data.positions[indexA].c = cA;
        data.positions[indexA].a = aA;
        data.positions[indexB].c = cB;
        data.positions[indexB].a = aB;
        data.positions[indexC].c = cC;
        data.positions[indexC].a = aC;
        data.positions[indexD].c = cD;
        data.positions[indexD].a = aD;
        return true;                                                    // linearError stays 0
    }

    void RopeInit(const SolverData& data) {                             // b2ropejoint.d:165-245
        LoadBodies();
        Vec2 cA = data.positions[indexA].c;
        f32 aA = data.positions[indexA].a;
        Vec2 vA = data.velocities[indexA].v;
        f32 wA = data.velocities[indexA].w;
        Vec2 cB = data.positions[indexB].c;
        f32 aB = data.positions[indexB].a;
        Vec2 vB = data.velocities[indexB].v;
        f32 wB = data.velocities[indexB].w;
        Rot qA(aA), qB(aB);
        rA = Mul(qA, localAnchorA - localCenterA);
        rB = Mul(qB, localAnchorB - localCenterB);
        u = ((cB + rB) - cA) - rA;
        curLength = u.Length();
        f32 C = curLength - length;
        limitState = C > 0.0f ? kAtUpperLimit : kInactiveLimit;
        if (curLength > kLinearSlop) {
            u *= 1.0f / curLength;
        } else {
            u.SetZero();
            distMass = 0.0f;
            impulse.x = 0.0f;
            return;
        }
        f32 crA = Cross(rA, u);
        f32 crB = Cross(rB, u);
        f32 invMass = ((invMassA + (invIA * crA) * crA) + invMassB) + (invIB * crB) * crB;
        distMass = invMass != 0.0f ? 1.0f / invMass : 0.0f;
        if (data.step.warmStarting) {
            impulse.x *= data.step.dtRatio;
            Vec2 P = impulse.x * u;
            vA -= invMassA * P;
            wA -= invIA * Cross(rA, P);
            vB += invMassB * P;
            wB += invIB * Cross(rB, P);
        } else {
            impulse.x = 0.0f;
        }
        data.velocities[indexA].v = vA;
        data.velocities[indexA].w = wA;
        data.velocities[indexB].v = vB;
        data.velocities[indexB].w = wB;
    }

    void RopeSolveVelocity(const SolverData& data) {                    // b2ropejoint.d:247-281
        Vec2 vA = data.velocities[indexA].v;
        f32 wA = data.velocities[indexA].w;
        Vec2 vB = data.velocities[indexB].v;
        f32 wB = data.velocities[indexB].w;
        Vec2 vpA = vA + Cross(wA, rA);
        Vec2 vpB = vB + Cross(wB, rB);
        f32 C = curLength - length;
        f32 Cdot = Dot(u, vpB - vpA);
        if (C < 0.0f) Cdot += data.step.inv_dt * C;                      // predictive constraint
        f32 imp = -distMass * Cdot;
        f32 oldImpulse = impulse.x;
        impulse.x = Min(0.0f, impulse.x + imp);
        imp = impulse.x - oldImpulse;
        Vec2 P = imp * u;
        vA -= invMassA * P;
        wA -= invIA * Cross(rA, P);
        vB += invMassB * P;
        wB += invIB * Cross(rB, P);
        data.velocities[indexA].v = vA;
        data.velocities[indexA].w = wA;
        data.velocities[indexB].v = vB;
        data.velocities[indexB].w = wB;
    }

    bool RopeSolvePosition(const SolverData& data) {                    // b2ropejoint.d:283-317
        Vec2 cA = data.positions[indexA].c;
        f32 aA = data.positions[indexA].a;
        Vec2 cB = data.positions[indexB].c;
        f32 aB = data.positions[indexB].a;
        Rot qA(aA), qB(aB);
        Vec2 rA_ = Mul(qA, localAnchorA - localCenterA);
        Vec2 rB_ = Mul(qB, localAnchorB - localCenterB);
        Vec2 d = ((cB + rB_) - cA) - rA_;
        f32 len = d.Normalize();
        f32 C = Clamp(len - length, 0.0f, kMaxLinearCorrection);
        f32 imp = -distMass * C;
        Vec2 P = imp * d;
        cA -= invMassA * P;
        aA -= invIA * Cross(rA_, P);
        cB += invMassB * P;
        aB += invIB * Cross(rB_, P);
        data.positions[indexA].c = cA;
        data.positions[indexA].a = aA;
        data.positions[indexB].c = cB;
        data.positions[indexB].a = aB;
        return len - length < kLinearSlop;
    }

    // b2FrictionJoint (b2frictionjoint.d:178-315) and b2MotorJoint (b2motorjoint.d:223-366): the
    // same 2x2 linear and 1x1 angular blocks with force / torque caps; the motor's anchors are
    // the bodies' origins and it drives towards an offset with a correction factor
    void FrictionMotorInit(const SolverData& data) {
        LoadBodies();
        Vec2 cA = data.positions[indexA].c;
        f32 aA = data.positions[indexA].a;
        Vec2 vA = data.velocities[indexA].v;
        f32 wA = data.velocities[indexA].w;
        Vec2 cB = data.positions[indexB].c;
        f32 aB = data.positions[indexB].a;
        Vec2 vB = data.velocities[indexB].v;
        f32 wB = data.velocities[indexB].w;
        Rot qA(aA), qB(aB);
        if (type == kMotorJoint) {
            rA = Mul(qA, -localCenterA);
            rB = Mul(qB, -localCenterB);
        } else {
            rA = Mul(qA, localAnchorA - localCenterA);
            rB = Mul(qB, localAnchorB - localCenterB);
        }
        f32 mA = invMassA, mB = invMassB, iA = invIA, iB = invIB;
        Mat22 K;
        K.ex.x = ((mA + mB) + (iA * rA.y) * rA.y) + (iB * rB.y) * rB.y;
        K.ex.y = ((-iA) * rA.x) * rA.y - (iB * rB.x) * rB.y;
        K.ey.x = K.ex.y;
        K.ey.y = ((mA + mB) + (iA * rA.x) * rA.x) + (iB * rB.x) * rB.x;
        linearMass = K.GetInverse();
        angularMass = iA + iB;
        if (angularMass > 0.0f) angularMass = 1.0f / angularMass;
        if (type == kMotorJoint) {
            linearError = ((((cB + rB) - cA) - rA) - Mul(qA, linearOffset));
            angularError = (aB - aA) - angularOffset;
        }
        if (data.step.warmStarting) {
            impulse.x *= data.step.dtRatio;
            impulse.y *= data.step.dtRatio;
            impulse.z *= data.step.dtRatio;
            Vec2 P(impulse.x, impulse.y);
            vA -= mA * P;
            wA -= iA * (Cross(rA, P) + impulse.z);
            vB += mB * P;
            wB += iB * (Cross(rB, P) + impulse.z);
        } else {
            impulse.SetZero();
        }
        data.velocities[indexA].v = vA;
        data.velocities[indexA].w = wA;
        data.velocities[indexB].v = vB;
        data.velocities[indexB].w = wB;
    }

    void FrictionMotorSolveVelocity(const SolverData& data) {
        Vec2 vA = data.velocities[indexA].v;
        f32 wA = data.velocities[indexA].w;
        Vec2 vB = data.velocities[indexB].v;
        f32 wB = data.velocities[indexB].w;
        f32 mA = invMassA, mB = invMassB, iA = invIA, iB = invIB;
        f32 h = data.step.dt, inv_h = data.step.inv_dt;
        {
            f32 Cdot = wB - wA;
            if (type == kMotorJoint) Cdot = Cdot + (inv_h * correctionFactor) * angularError;
            f32 imp = -angularMass * Cdot;
            f32 oldImpulse = impulse.z;
            f32 maxImpulse = h * maxTorque;
            impulse.z = Clamp(impulse.z + imp, -maxImpulse, maxImpulse);
            imp = impulse.z - oldImpulse;
            wA -= iA * imp;
            wB += iB * imp;
        }
        {
            Vec2 Cdot = ((vB + Cross(wB, rB)) - vA) - Cross(wA, rA);
            if (type == kMotorJoint) Cdot = Cdot + (inv_h * correctionFactor) * linearError;
            Vec2 imp = -Mul(linearMass, Cdot);
            Vec2 oldImpulse(impulse.x, impulse.y);
            Vec2 li(impulse.x + imp.x, impulse.y + imp.y);
            f32 maxImpulse = h * maxForce;
            if (li.LengthSquared() > maxImpulse * maxImpulse) {
                li.Normalize();
                li *= maxImpulse;
            }
            impulse.x = li.x;
            impulse.y = li.y;
            imp = li - oldImpulse;
            vA -= mA * imp;
            wA -= iA * Cross(rA, imp);
            vB += mB * imp;
            wB += iB * Cross(rB, imp);
        }
        data.velocities[indexA].v = vA;
        data.velocities[indexA].w = wA;
        data.velocities[indexB].v = vB;
        data.velocities[indexB].w = wB;
    }

    void WheelInit(const SolverData& data) {                            // b2wheeljoint.d:302-443
        LoadBodies();
        f32 mA = invMassA, mB = invMassB, iA = invIA, iB = invIB;
        Vec2 cA = data.positions[indexA].c;
        f32 aA = data.positions[indexA].a;
        Vec2 vA = data.velocities[indexA].v;
        f32 wA = data.velocities[indexA].w;
        Vec2 cB = data.positions[indexB].c;
        f32 aB = data.positions[indexB].a;
        Vec2 vB = data.velocities[indexB].v;
        f32 wB = data.velocities[indexB].w;
        Rot qA(aA), qB(aB);
        Vec2 rA_ = Mul(qA, localAnchorA - localCenterA);
        Vec2 rB_ = Mul(qB, localAnchorB - localCenterB);
        Vec2 d = ((cB + rB_) - cA) - rA_;
        ay = Mul(qA, localYAxisA);                                      // point to line
        sAy = Cross(d + rA_, ay);
        sBy = Cross(rB_, ay);
        wheelMass = ((mA + mB) + (iA * sAy) * sAy) + (iB * sBy) * sBy;
        if (wheelMass > 0.0f) wheelMass = 1.0f / wheelMass;
        springMass = 0.0f;                                              // spring
        bias = 0.0f;
        gamma = 0.0f;
        if (frequencyHz > 0.0f) {
            ax = Mul(qA, localXAxisA);
            sAx = Cross(d + rA_, ax);
            sBx = Cross(rB_, ax);
            f32 invMass = ((mA + mB) + (iA * sAx) * sAx) + (iB * sBx) * sBx;
            if (invMass > 0.0f) {
                springMass = 1.0f / invMass;
                f32 C = Dot(d, ax);
                f32 omega = (2.0f * kPi) * frequencyHz;
                f32 d2 = ((2.0f * springMass) * dampingRatio) * omega;
                f32 k = (springMass * omega) * omega;
                f32 h = data.step.dt;
                gamma = h * (d2 + h * k);
                if (gamma > 0.0f) gamma = 1.0f / gamma;
                bias = ((C * h) * k) * gamma;
                springMass = invMass + gamma;
                if (springMass > 0.0f) springMass = 1.0f / springMass;
            }
        } else {
            impulse.y = 0.0f;
        }
        if (enableMotor) {                                              // rotational motor
            motorMass = iA + iB;
            if (motorMass > 0.0f) motorMass = 1.0f / motorMass;
        } else {
            motorMass = 0.0f;
            motorImpulse = 0.0f;
        }
        if (data.step.warmStarting) {
            impulse.x *= data.step.dtRatio;
            impulse.y *= data.step.dtRatio;
            motorImpulse *= data.step.dtRatio;
            Vec2 P = impulse.x * ay + impulse.y * ax;
            f32 LA = (impulse.x * sAy + impulse.y * sAx) + motorImpulse;
            f32 LB = (impulse.x * sBy + impulse.y * sBx) + motorImpulse;
            vA -= invMassA * P;
            wA -= invIA * LA;
            vB += invMassB * P;
            wB += invIB * LB;
        } else {
            impulse.x = 0.0f;
            impulse.y = 0.0f;
            motorImpulse = 0.0f;
        }
        data.velocities[indexA].v = vA;
        data.velocities[indexA].w = wA;
        data.velocities[indexB].v = vB;
        data.velocities[indexB].w = wB;
    }

    void WheelSolveVelocity(const SolverData& data) {                   // b2wheeljoint.d:445-507
        f32 mA = invMassA, mB = invMassB, iA = invIA, iB = invIB;
        Vec2 vA = data.velocities[indexA].v;
        f32 wA = data.velocities[indexA].w;
        Vec2 vB = data.velocities[indexB].v;
        f32 wB = data.velocities[indexB].w;
        {                                                               // spring
            f32 Cdot = (Dot(ax, vB - vA) + sBx * wB) - sAx * wA;
            f32 imp = -springMass * ((Cdot + bias) + gamma * impulse.y);
            impulse.y += imp;
            Vec2 P = imp * ax;
            f32 LA = imp * sAx, LB = imp * sBx;
            vA -= mA * P;
            wA -= iA * LA;
            vB += mB * P;
            wB += iB * LB;
        }
        {                                                               // rotational motor
            f32 Cdot = (wB - wA) - motorSpeed;
            f32 imp = -motorMass * Cdot;
            f32 oldImpulse = motorImpulse;
            f32 maxImpulse = data.step.dt * maxMotorTorque;
            motorImpulse = Clamp(motorImpulse + imp, -maxImpulse, maxImpulse);
            imp = motorImpulse - oldImpulse;
            wA -= iA * imp;
            wB += iB * imp;
        }
        {                                                               // point to line
            f32 Cdot = (Dot(ay, vB - vA) + sBy * wB) - sAy * wA;
            f32 imp = -wheelMass * Cdot;
            impulse.x += imp;
            Vec2 P = imp * ay;
            f32 LA = imp * sAy, LB = imp * sBy;
            vA -= mA * P;
            wA -= iA * LA;
            vB += mB * P;
            wB += iB * LB;
        }
        data.velocities[indexA].v = vA;
        data.velocities[indexA].w = wA;
        data.velocities[indexB].v = vB;
        data.velocities[indexB].w = wB;
    }

    bool WheelSolvePosition(const SolverData& data) {                   // b2wheeljoint.d:509-553
        Vec2 cA = data.positions[indexA].c;
        f32 aA = data.positions[indexA].a;
        Vec2 cB = data.positions[indexB].c;
        f32 aB = data.positions[indexB].a;
        Rot qA(aA), qB(aB);
        Vec2 rA_ = Mul(qA, localAnchorA - localCenterA);
        Vec2 rB_ = Mul(qB, localAnchorB - localCenterB);
        Vec2 d = ((cB - cA) + rB_) - rA_;
        Vec2 ay_ = Mul(qA, localYAxisA);
        f32 sAy_ = Cross(d + rA_, ay_);
        f32 sBy_ = Cross(rB_, ay_);
        f32 C = Dot(d, ay_);
        // the effective mass uses the velocity pass's sAy / sBy, as the reference does
        f32 k = ((invMassA + invMassB) + (invIA * sAy) * sAy) + (invIB * sBy) * sBy;
        f32 imp = k != 0.0f ? -C / k : 0.0f;
        Vec2 P = imp * ay_;
        f32 LA = imp * sAy_, LB = imp * sBy_;
        cA -= invMassA * P;
        aA -= invIA * LA;
        cB += invMassB * P;
        aB += invIB * LB;
        data.positions[indexA].c = cA;
        data.positions[indexA].a = aA;
        data.positions[indexB].c = cB;
        data.positions[indexB].a = aB;
        return Abs(C) <= kLinearSlop;
    }

    void PrismaticInit(const SolverData& data) {                        // b2prismaticjoint.d:391-533
        LoadBodies();
        Vec2 cA = data.positions[indexA].c;
        f32 aA = data.positions[indexA].a;
        Vec2 vA = data.velocities[indexA].v;
        f32 wA = data.velocities[indexA].w;
        Vec2 cB = data.positions[indexB].c;
        f32 aB = data.positions[indexB].a;
        Vec2 vB = data.velocities[indexB].v;
        f32 wB = data.velocities[indexB].w;
        Rot qA(aA), qB(aB);
        Vec2 rA_ = Mul(qA, localAnchorA - localCenterA);
        Vec2 rB_ = Mul(qB, localAnchorB - localCenterB);
        Vec2 d = ((cB - cA) + rB_) - rA_;
        f32 mA = invMassA, mB = invMassB, iA = invIA, iB = invIB;
        axis = Mul(qA, localXAxisA);                                    // motor Jacobian and effective mass
        a1 = Cross(d + rA_, axis);
        a2 = Cross(rB_, axis);
        motorMass = ((mA + mB) + (iA * a1) * a1) + (iB * a2) * a2;
        if (motorMass > 0.0f) motorMass = 1.0f / motorMass;
        perp = Mul(qA, localYAxisA);                                    // prismatic constraint
        s1 = Cross(d + rA_, perp);
        s2 = Cross(rB_, perp);
        f32 k11 = ((mA + mB) + (iA * s1) * s1) + (iB * s2) * s2;
        f32 k12 = iA * s1 + iB * s2;
        f32 k13 = (iA * s1) * a1 + (iB * s2) * a2;
        f32 k22 = iA + iB;
        if (k22 == 0.0f) k22 = 1.0f;                                    // fixed rotation
        f32 k23 = iA * a1 + iB * a2;
        f32 k33 = ((mA + mB) + (iA * a1) * a1) + (iB * a2) * a2;
        massM.ex = Vec3(k11, k12, k13);
        massM.ey = Vec3(k12, k22, k23);
        massM.ez = Vec3(k13, k23, k33);
        if (enableLimit) {                                              // limit state
            f32 jointTranslation = Dot(axis, d);
            if (Abs(upperTranslation - lowerTranslation) < 2.0f * kLinearSlop) {
                limitState = kEqualLimits;
            } else if (jointTranslation <= lowerTranslation) {
                if (limitState != kAtLowerLimit) { limitState = kAtLowerLimit; impulse.z = 0.0f; }
            } else if (jointTranslation >= upperTranslation) {
                if (limitState != kAtUpperLimit) { limitState = kAtUpperLimit; impulse.z = 0.0f; }
            } else {
                limitState = kInactiveLimit;
                impulse.z = 0.0f;
            }
        } else {
            limitState = kInactiveLimit;
            impulse.z = 0.0f;
        }
        if (!enableMotor) motorImpulse = 0.0f;
        if (data.step.warmStarting) {
            impulse *= data.step.dtRatio;
            motorImpulse *= data.step.dtRatio;
            Vec2 P = impulse.x * perp + (motorImpulse + impulse.z) * axis;
            f32 LA = (impulse.x * s1 + impulse.y) + (motorImpulse + impulse.z) * a1;
            f32 LB = (impulse.x * s2 + impulse.y) + (motorImpulse + impulse.z) * a2;
            vA -= mA * P;
            wA -= iA * LA;
            vB += mB * P;
            wB += iB * LB;
        } else {
            impulse.SetZero();
            motorImpulse = 0.0f;
        }
        data.velocities[indexA].v = vA;
        data.velocities[indexA].w = wA;
        data.velocities[indexB].v = vB;
        data.velocities[indexB].w = wB;
    }

    void PrismaticSolveVelocity(const SolverData& data) {               // b2prismaticjoint.d:535-630
        Vec2 vA = data.velocities[indexA].v;
        f32 wA = data.velocities[indexA].w;
        Vec2 vB = data.velocities[indexB].v;
        f32 wB = data.velocities[indexB].w;
        f32 mA = invMassA, mB = invMassB, iA = invIA, iB = invIB;
        if (enableMotor && limitState != kEqualLimits) {                // motor
            f32 Cdot = (Dot(axis, vB - vA) + a2 * wB) - a1 * wA;
            f32 imp = motorMass * (motorSpeed - Cdot);
            f32 oldImpulse = motorImpulse;
            f32 maxImpulse = data.step.dt * maxMotorForce;
            motorImpulse = Clamp(motorImpulse + imp, -maxImpulse, maxImpulse);
            imp = motorImpulse - oldImpulse;
            Vec2 P = imp * axis;
            f32 LA = imp * a1, LB = imp * a2;
            vA -= mA * P;
            wA -= iA * LA;
            vB += mB * P;
            wB += iB * LB;
        }
        Vec2 Cdot1;
        Cdot1.x = (Dot(perp, vB - vA) + s2 * wB) - s1 * wA;
        Cdot1.y = wB - wA;
        if (enableLimit && limitState != kInactiveLimit) {              // prismatic and limit together
            f32 Cdot2 = (Dot(axis, vB - vA) + a2 * wB) - a1 * wA;
            Vec3 Cdot(Cdot1.x, Cdot1.y, Cdot2);
            Vec3 f1 = impulse;
            Vec3 df = massM.Solve33(-Cdot);
            impulse += df;
            if (limitState == kAtLowerLimit) impulse.z = Max(impulse.z, 0.0f);
            else if (limitState == kAtUpperLimit) impulse.z = Min(impulse.z, 0.0f);
            // f2(1:2) = invK(1:2,1:2) * (-Cdot(1:2) - K(1:2,3) * (f2(3) - f1(3))) + f1(1:2)
            Vec2 b = -Cdot1 - (impulse.z - f1.z) * Vec2(massM.ez.x, massM.ez.y);
            Vec2 f2r = massM.Solve22(b) + Vec2(f1.x, f1.y);
            impulse.x = f2r.x;
            impulse.y = f2r.y;
            df = Vec3(impulse.x - f1.x, impulse.y - f1.y, impulse.z - f1.z);
            Vec2 P = df.x * perp + df.z * axis;
            f32 LA = (df.x * s1 + df.y) + df.z * a1;
            f32 LB = (df.x * s2 + df.y) + df.z * a2;
            vA -= mA * P;
            wA -= iA * LA;
            vB += mB * P;
            wB += iB * LB;
        } else {                                                        // prismatic only
            Vec2 df = massM.Solve22(-Cdot1);
            impulse.x += df.x;
            impulse.y += df.y;
            Vec2 P = df.x * perp;
            f32 LA = df.x * s1 + df.y;
            f32 LB = df.x * s2 + df.y;
            vA -= mA * P;
            wA -= iA * LA;
            vB += mB * P;
            wB += iB * LB;
        }
        data.velocities[indexA].v = vA;
        data.velocities[indexA].w = wA;
        data.velocities[indexB].v = vB;
        data.velocities[indexB].w = wB;
    }

    bool PrismaticSolvePosition(const SolverData& data) {               // b2prismaticjoint.d:632-757
        Vec2 cA = data.positions[indexA].c;
        f32 aA = data.positions[indexA].a;
        Vec2 cB = data.positions[indexB].c;
        f32 aB = data.positions[indexB].a;
        Rot qA(aA), qB(aB);
        f32 mA = invMassA, mB = invMassB, iA = invIA, iB = invIB;
        Vec2 rA_ = Mul(qA, localAnchorA - localCenterA);
        Vec2 rB_ = Mul(qB, localAnchorB - localCenterB);
        Vec2 d = ((cB + rB_) - cA) - rA_;
        Vec2 axis_ = Mul(qA, localXAxisA);
        f32 a1_ = Cross(d + rA_, axis_);
        f32 a2_ = Cross(rB_, axis_);
        Vec2 perp_ = Mul(qA, localYAxisA);
        f32 s1_ = Cross(d + rA_, perp_);
        f32 s2_ = Cross(rB_, perp_);
        Vec3 imp;
        Vec2 C1;
        C1.x = Dot(perp_, d);
        C1.y = (aB - aA) - referenceAngle;
        f32 linearError = Abs(C1.x);
        f32 angularError = Abs(C1.y);
        bool active = false;
        f32 C2 = 0.0f;
        if (enableLimit) {
            f32 translation = Dot(axis_, d);
            if (Abs(upperTranslation - lowerTranslation) < 2.0f * kLinearSlop) {
                C2 = Clamp(translation, -kMaxLinearCorrection, kMaxLinearCorrection);
                linearError = Max(linearError, Abs(translation));
                active = true;
            } else if (translation <= lowerTranslation) {
                C2 = Clamp((translation - lowerTranslation) + kLinearSlop, -kMaxLinearCorrection, 0.0f);
                linearError = Max(linearError, lowerTranslation - translation);
                active = true;
            } else if (translation >= upperTranslation) {
                C2 = Clamp((translation - upperTranslation) - kLinearSlop, 0.0f, kMaxLinearCorrection);
                linearError = Max(linearError, translation - upperTranslation);
                active = true;
            }
        }
        if (active) {
            f32 k11 = ((mA + mB) + (iA * s1_) * s1_) + (iB * s2_) * s2_;
            f32 k12 = iA * s1_ + iB * s2_;
            f32 k13 = (iA * s1_) * a1_ + (iB * s2_) * a2_;
            f32 k22 = iA + iB;
            if (k22 == 0.0f) k22 = 1.0f;
            f32 k23 = iA * a1_ + iB * a2_;
            f32 k33 = ((mA + mB) + (iA * a1_) * a1_) + (iB * a2_) * a2_;
            Mat33 K;
            K.ex = Vec3(k11, k12, k13);
            K.ey = Vec3(k12, k22, k23);
            K.ez = Vec3(k13, k23, k33);
            imp = K.Solve33(-Vec3(C1.x, C1.y, C2));
        } else {
            f32 k11 = ((mA + mB) + (iA * s1_) * s1_) + (iB * s2_) * s2_;
            f32 k12 = iA * s1_ + iB * s2_;
            f32 k22 = iA + iB;
            if (k22 == 0.0f) k22 = 1.0f;
            Mat33 K;
            K.ex = Vec3(k11, k12, 0.0f);
            K.ey = Vec3(k12, k22, 0.0f);
            Vec2 impulse1 = K.Solve22(-C1);                             // b2Mat22.Solve: the same 2x2 solve
            imp = Vec3(impulse1.x, impulse1.y, 0.0f);
        }
        Vec2 P = imp.x * perp_ + imp.z * axis_;
        f32 LA = (imp.x * s1_ + imp.y) + imp.z * a1_;
        f32 LB = (imp.x * s2_ + imp.y) + imp.z * a2_;
        cA -= mA * P;
        aA -= iA * LA;
        cB += mB * P;
        aB += iB * LB;
        data.positions[indexA].c = cA;
        data.positions[indexA].a = aA;
        data.positions[indexB].c = cB;
        data.positions[indexB].a = aB;
        return linearError <= kLinearSlop && angularError <= kAngularSlop;
    }

    void PulleyInit(const SolverData& data) {                           // b2pulleyjoint.d:181-262
        LoadBodies();
        Vec2 cA = data.positions[indexA].c;
        f32 aA = data.positions[indexA].a;
        Vec2 vA = data.velocities[indexA].v;
        f32 wA = data.velocities[indexA].w;
        Vec2 cB = data.positions[indexB].c;
        f32 aB = data.positions[indexB].a;
        Vec2 vB = data.velocities[indexB].v;
        f32 wB = data.velocities[indexB].w;
        Rot qA(aA), qB(aB);
        rA = Mul(qA, localAnchorA - localCenterA);
        rB = Mul(qB, localAnchorB - localCenterB);
        uA = (cA + rA) - groundAnchorA;                                 // the pulley axes
        uB = (cB + rB) - groundAnchorB;
        f32 lengthA = uA.Length(), lengthB = uB.Length();
        if (lengthA > 10.0f * kLinearSlop) uA *= 1.0f / lengthA; else uA.SetZero();
        if (lengthB > 10.0f * kLinearSlop) uB *= 1.0f / lengthB; else uB.SetZero();
        f32 ruA = Cross(rA, uA), ruB = Cross(rB, uB);
        f32 mA = invMassA + (invIA * ruA) * ruA;
        f32 mB = invMassB + (invIB * ruB) * ruB;
        distMass = mA + (ratio * ratio) * mB;
        if (distMass > 0.0f) distMass = 1.0f / distMass;
        if (data.step.warmStarting) {
            impulse.x *= data.step.dtRatio;
            Vec2 PA = (-impulse.x) * uA;
            Vec2 PB = ((-ratio) * impulse.x) * uB;
            vA += invMassA * PA;
            wA += invIA * Cross(rA, PA);
            vB += invMassB * PB;
            wB += invIB * Cross(rB, PB);
        } else {
            impulse.x = 0.0f;
        }
        data.velocities[indexA].v = vA;
        data.velocities[indexA].w = wA;
        data.velocities[indexB].v = vB;
        data.velocities[indexB].w = wB;
    }

    void PulleySolveVelocity(const SolverData& data) {                  // b2pulleyjoint.d:264-289
        Vec2 vA = data.velocities[indexA].v;
        f32 wA = data.velocities[indexA].w;
        Vec2 vB = data.velocities[indexB].v;
        f32 wB = data.velocities[indexB].w;
        Vec2 vpA = vA + Cross(wA, rA);
        Vec2 vpB = vB + Cross(wB, rB);
        f32 Cdot = (-Dot(uA, vpA)) - ratio * Dot(uB, vpB);
        f32 imp = -distMass * Cdot;
        impulse.x += imp;
        Vec2 PA = (-imp) * uA;
        Vec2 PB = ((-ratio) * imp) * uB;
        vA += invMassA * PA;
        wA += invIA * Cross(rA, PA);
        vB += invMassB * PB;
        wB += invIB * Cross(rB, PB);
        data.velocities[indexA].v = vA;
        data.velocities[indexA].w = wA;
        data.velocities[indexB].v = vB;
        data.velocities[indexB].w = wB;
    }

    bool PulleySolvePosition(const SolverData& data) {                  // b2pulleyjoint.d:291-350
        Vec2 cA = data.positions[indexA].c;
        f32 aA = data.positions[indexA].a;
        Vec2 cB = data.positions[indexB].c;
        f32 aB = data.positions[indexB].a;
        Rot qA(aA), qB(aB);
        Vec2 rA_ = Mul(qA, localAnchorA - localCenterA);
        Vec2 rB_ = Mul(qB, localAnchorB - localCenterB);
        Vec2 uA_ = (cA + rA_) - groundAnchorA;
        Vec2 uB_ = (cB + rB_) - groundAnchorB;
        f32 lengthA = uA_.Length(), lengthB = uB_.Length();
        if (lengthA > 10.0f * kLinearSlop) uA_ *= 1.0f / lengthA; else uA_.SetZero();
        if (lengthB > 10.0f * kLinearSlop) uB_ *= 1.0f / lengthB; else uB_.SetZero();
        f32 ruA = Cross(rA_, uA_), ruB = Cross(rB_, uB_);
        f32 mA = invMassA + (invIA * ruA) * ruA;
        f32 mB = invMassB + (invIB * ruB) * ruB;
        f32 mass = mA + (ratio * ratio) * mB;
        if (mass > 0.0f) mass = 1.0f / mass;
        f32 C = (constant - lengthA) - ratio * lengthB;
        f32 linearError = Abs(C);
        f32 imp = -mass * C;
        Vec2 PA = (-imp) * uA_;
        Vec2 PB = ((-ratio) * imp) * uB_;
        cA += invMassA * PA;
        aA += invIA * Cross(rA_, PA);
        cB += invMassB * PB;
        aB += invIB * Cross(rB_, PB);
        data.positions[indexA].c = cA;
        data.positions[indexA].a = aA;
        data.positions[indexB].c = cB;
        data.positions[indexB].a = aB;
        return linearError < kLinearSlop;
    }

    void MouseInit(const SolverData& data) {                            // b2mousejoint.d:132-192 (body B only)
        indexB = bodyB->islandIndex;
        localCenterB = bodyB->sweep.localCenter;
        invMassB = bodyB->invMass;
        invIB = bodyB->invI;
        Vec2 cB = data.positions[indexB].c;
        f32 aB = data.positions[indexB].a;
        Vec2 vB = data.velocities[indexB].v;
        f32 wB = data.velocities[indexB].w;
        Rot qB(aB);
        f32 mass = bodyB->mass;
        f32 omega = (2.0f * kPi) * frequencyHz;                         // frequency
        f32 d = ((2.0f * mass) * dampingRatio) * omega;                 // damping coefficient
        f32 k = mass * (omega * omega);                                 // spring stiffness
        f32 h = data.step.dt;
        gamma = h * (d + h * k);
        if (gamma != 0.0f) gamma = 1.0f / gamma;
        beta = (h * k) * gamma;
        rB = Mul(qB, localAnchorB - localCenterB);
        Mat22 K;
        K.ex.x = (invMassB + (invIB * rB.y) * rB.y) + gamma;
        K.ex.y = ((-invIB) * rB.x) * rB.y;
        K.ey.x = K.ex.y;
        K.ey.y = (invMassB + (invIB * rB.x) * rB.x) + gamma;
        linearMass = K.GetInverse();
        mouseC = (cB + rB) - targetA;
        mouseC *= beta;
        wB *= 0.98f;                                                    // cheat with some damping
        if (data.step.warmStarting) {
            impulse.x *= data.step.dtRatio;
            impulse.y *= data.step.dtRatio;
            Vec2 I(impulse.x, impulse.y);
            vB += invMassB * I;
            wB += invIB * Cross(rB, I);
        } else {
            impulse.SetZero();
        }
        data.velocities[indexB].v = vB;
        data.velocities[indexB].w = wB;
    }

    void MouseSolveVelocity(const SolverData& data) {                   // b2mousejoint.d:194-220
        Vec2 vB = data.velocities[indexB].v;
        f32 wB = data.velocities[indexB].w;
        Vec2 Cdot = vB + Cross(wB, rB);
        Vec2 I(impulse.x, impulse.y);
        Vec2 imp = Mul(linearMass, -((Cdot + mouseC) + gamma * I));
        Vec2 oldImpulse = I;
        I += imp;
        f32 maxImpulse = data.step.dt * maxForce;
        if (I.LengthSquared() > maxImpulse * maxImpulse) I *= maxImpulse / I.Length();
        impulse.x = I.x;
        impulse.y = I.y;
        imp = I - oldImpulse;
        vB += invMassB * imp;
        wB += invIB * Cross(rB, imp);
        data.velocities[indexB].v = vB;
        data.velocities[indexB].w = wB;
    }

    // the weld joint's K (b2weldjoint.d:229-238 and 387-396)
    static Mat33 WeldK(f32 mA, f32 mB, f32 iA, f32 iB, Vec2 ra, Vec2 rb) {
        Mat33 K;
        K.ex.x = ((mA + mB) + (ra.y * ra.y) * iA) + (rb.y * rb.y) * iB;
        K.ey.x = ((-ra.y) * ra.x) * iA - (rb.y * rb.x) * iB;
        K.ez.x = (-ra.y) * iA - rb.y * iB;
        K.ex.y = K.ey.x;
        K.ey.y = ((mA + mB) + (ra.x * ra.x) * iA) + (rb.x * rb.x) * iB;
        K.ez.y = ra.x * iA + rb.x * iB;
        K.ex.z = K.ez.x;
        K.ey.z = K.ez.y;
        K.ez.z = iA + iB;
        return K;
    }

    void WeldInit(const SolverData& data) {                             // b2weldjoint.d:196-306
        LoadBodies();
        f32 aA = data.positions[indexA].a;
        Vec2 vA = data.velocities[indexA].v;
        f32 wA = data.velocities[indexA].w;
        f32 aB = data.positions[indexB].a;
        Vec2 vB = data.velocities[indexB].v;
        f32 wB = data.velocities[indexB].w;
        Rot qA(aA), qB(aB);
        rA = Mul(qA, localAnchorA - localCenterA);
        rB = Mul(qB, localAnchorB - localCenterB);
        f32 mA = invMassA, mB = invMassB, iA = invIA, iB = invIB;
        Mat33 K = WeldK(mA, mB, iA, iB, rA, rB);
        if (frequencyHz > 0.0f) {
            K.GetInverse22(&massM);
            f32 invM = iA + iB;
            f32 m = invM > 0.0f ? 1.0f / invM : 0.0f;
            f32 C = (aB - aA) - referenceAngle;
            f32 omega = (2.0f * kPi) * frequencyHz;
            f32 d = ((2.0f * m) * dampingRatio) * omega;
            f32 k = (m * omega) * omega;
            f32 h = data.step.dt;
            gamma = h * (d + h * k);
            gamma = gamma != 0.0f ? 1.0f / gamma : 0.0f;
            bias = ((C * h) * k) * gamma;
            invM += gamma;
            massM.ez.z = invM != 0.0f ? 1.0f / invM : 0.0f;
        } else if (K.ez.z == 0.0f) {
            K.GetInverse22(&massM);
            gamma = 0.0f;
            bias = 0.0f;
        } else {
            K.GetSymInverse33(&massM);
            gamma = 0.0f;
            bias = 0.0f;
        }
        if (data.step.warmStarting) {
            impulse *= data.step.dtRatio;
            Vec2 P(impulse.x, impulse.y);
            vA -= mA * P;
            wA -= iA * (Cross(rA, P) + impulse.z);
            vB += mB * P;
            wB += iB * (Cross(rB, P) + impulse.z);
        } else {
            impulse.SetZero();
        }
        data.velocities[indexA].v = vA;
        data.velocities[indexA].w = wA;
        data.velocities[indexB].v = vB;
        data.velocities[indexB].w = wB;
    }

    void WeldSolveVelocity(const SolverData& data) {                    // b2weldjoint.d:308-364
        Vec2 vA = data.velocities[indexA].v;
        f32 wA = data.velocities[indexA].w;
        Vec2 vB = data.velocities[indexB].v;
        f32 wB = data.velocities[indexB].w;
        f32 mA = invMassA, mB = invMassB, iA = invIA, iB = invIB;
        if (frequencyHz > 0.0f) {
            f32 Cdot2 = wB - wA;
            f32 impulse2 = -massM.ez.z * ((Cdot2 + bias) + gamma * impulse.z);
            impulse.z += impulse2;
            wA -= iA * impulse2;
            wB += iB * impulse2;
            Vec2 Cdot1 = ((vB + Cross(wB, rB)) - vA) - Cross(wA, rA);
            Vec2 impulse1 = -Mul22(massM, Cdot1);
            impulse.x += impulse1.x;
            impulse.y += impulse1.y;
            Vec2 P = impulse1;
            vA -= mA * P;
            wA -= iA * Cross(rA, P);
            vB += mB * P;
            wB += iB * Cross(rB, P);
        } else {
            Vec2 Cdot1 = ((vB + Cross(wB, rB)) - vA) - Cross(wA, rA);
            f32 Cdot2 = wB - wA;
            Vec3 Cdot(Cdot1.x, Cdot1.y, Cdot2);
            Vec3 imp = -Mul(massM, Cdot);
            impulse += imp;
            Vec2 P(imp.x, imp.y);
            vA -= mA * P;
            wA -= iA * (Cross(rA, P) + imp.z);
            vB += mB * P;
            wB += iB * (Cross(rB, P) + imp.z);
        }
        data.velocities[indexA].v = vA;
        data.velocities[indexA].w = wA;
        data.velocities[indexB].v = vB;
        data.velocities[indexB].w = wB;
    }

    bool WeldSolvePosition(const SolverData& data) {                    // b2weldjoint.d:366-444
        Vec2 cA = data.positions[indexA].c;
        f32 aA = data.positions[indexA].a;
        Vec2 cB = data.positions[indexB].c;
        f32 aB = data.positions[indexB].a;
        Rot qA(aA), qB(aB);
        f32 mA = invMassA, mB = invMassB, iA = invIA, iB = invIB;
        Vec2 rA_ = Mul(qA, localAnchorA - localCenterA);
        Vec2 rB_ = Mul(qB, localAnchorB - localCenterB);
        f32 positionError = 0.0f, angularError = 0.0f;
        Mat33 K = WeldK(mA, mB, iA, iB, rA_, rB_);
        if (frequencyHz > 0.0f) {
            Vec2 C1 = ((cB + rB_) - cA) - rA_;
            positionError = C1.Length();
            angularError = 0.0f;
            Vec2 P = -K.Solve22(C1);
            cA -= mA * P;
            aA -= iA * Cross(rA_, P);
            cB += mB * P;
            aB += iB * Cross(rB_, P);
        } else {
            Vec2 C1 = ((cB + rB_) - cA) - rA_;
            f32 C2 = (aB - aA) - referenceAngle;
            positionError = C1.Length();
            angularError = Abs(C2);
            Vec3 C(C1.x, C1.y, C2);
            Vec3 imp;
            if (K.ez.z > 0.0f) {
                imp = -K.Solve33(C);
            } else {
                Vec2 imp2 = -K.Solve22(C1);
                imp = Vec3(imp2.x, imp2.y, 0.0f);
            }
            Vec2 P(imp.x, imp.y);
            cA -= mA * P;
            aA -= iA * (Cross(rA_, P) + imp.z);
            cB += mB * P;
            aB += iB * (Cross(rB_, P) + imp.z);
        }
        data.positions[indexA].c = cA;
        data.positions[indexA].a = aA;
        data.positions[indexB].c = cB;
        data.positions[indexB].a = aB;
        return positionError <= kLinearSlop && angularError <= kAngularSlop;
    }

    void DistanceInit(const SolverData& data) {                         // b2distancejoint.d:211-306
        indexA = bodyA->islandIndex;
        indexB = bodyB->islandIndex;
        localCenterA = bodyA->sweep.localCenter;
        localCenterB = bodyB->sweep.localCenter;
        invMassA = bodyA->invMass;
        invMassB = bodyB->invMass;
        invIA = bodyA->invI;
        invIB = bodyB->invI;
        Vec2 cA = data.positions[indexA].c;
        f32 aA = data.positions[indexA].a;
        Vec2 vA = data.velocities[indexA].v;
        f32 wA = data.velocities[indexA].w;
        Vec2 cB = data.positions[indexB].c;
        f32 aB = data.positions[indexB].a;
        Vec2 vB = data.velocities[indexB].v;
        f32 wB = data.velocities[indexB].w;
        Rot qA(aA), qB(aB);
        rA = Mul(qA, localAnchorA - localCenterA);
        rB = Mul(qB, localAnchorB - localCenterB);
        u = ((cB + rB) - cA) - rA;
        f32 len = u.Length();                                           // singularity: u = 0 below linearSlop
        if (len > kLinearSlop) u *= 1.0f / len;
        else u.Set(0.0f, 0.0f);
        f32 crAu = Cross(rA, u);
        f32 crBu = Cross(rB, u);
        f32 invMass = ((invMassA + (invIA * crAu) * crAu) + invMassB) + (invIB * crBu) * crBu;
        distMass = invMass != 0.0f ? 1.0f / invMass : 0.0f;
        if (frequencyHz > 0.0f) {
            f32 C = len - length;
            f32 omega = (2.0f * kPi) * frequencyHz;
            f32 d = ((2.0f * distMass) * dampingRatio) * omega;
            f32 k = (distMass * omega) * omega;
            f32 h = data.step.dt;
            gamma = h * (d + h * k);
            gamma = gamma != 0.0f ? 1.0f / gamma : 0.0f;
            bias = ((C * h) * k) * gamma;
            invMass += gamma;
            distMass = invMass != 0.0f ? 1.0f / invMass : 0.0f;
        } else {
            gamma = 0.0f;
            bias = 0.0f;
        }
        if (data.step.warmStarting) {
            impulse.x *= data.step.dtRatio;
            Vec2 P = impulse.x * u;
            vA -= invMassA * P;
            wA -= invIA * Cross(rA, P);
            vB += invMassB * P;
            wB += invIB * Cross(rB, P);
        } else {
            impulse.x = 0.0f;
        }
        data.velocities[indexA].v = vA;
        data.velocities[indexA].w = wA;
        data.velocities[indexB].v = vB;
        data.velocities[indexB].w = wB;
    }

    void DistanceSolveVelocity(const SolverData& data) {                // b2distancejoint.d:308-333
        Vec2 vA = data.velocities[indexA].v;
        f32 wA = data.velocities[indexA].w;
        Vec2 vB = data.velocities[indexB].v;
        f32 wB = data.velocities[indexB].w;
        Vec2 vpA = vA + Cross(wA, rA);
        Vec2 vpB = vB + Cross(wB, rB);
        f32 Cdot = Dot(u, vpB - vpA);
        f32 imp = -distMass * ((Cdot + bias) + gamma * impulse.x);
        impulse.x += imp;
        Vec2 P = imp * u;
        vA -= invMassA * P;
        wA -= invIA * Cross(rA, P);
        vB += invMassB * P;
        wB += invIB * Cross(rB, P);
        data.velocities[indexA].v = vA;
        data.velocities[indexA].w = wA;
        data.velocities[indexB].v = vB;
        data.velocities[indexB].w = wB;
    }

    bool DistanceSolvePosition(const SolverData& data) {                // b2distancejoint.d:335-372
        if (frequencyHz > 0.0f) return true;                            // soft: no position correction
        Vec2 cA = data.positions[indexA].c;
        f32 aA = data.positions[indexA].a;
        Vec2 cB = data.positions[indexB].c;
        f32 aB = data.positions[indexB].a;
        Rot qA(aA), qB(aB);
        Vec2 rA_ = Mul(qA, localAnchorA - localCenterA);
        Vec2 rB_ = Mul(qB, localAnchorB - localCenterB);
        Vec2 d = ((cB + rB_) - cA) - rA_;
        f32 len = d.Normalize();
        f32 C = len - length;
        C = Clamp(C, -kMaxLinearCorrection, kMaxLinearCorrection);
        f32 imp = -distMass * C;
        Vec2 P = imp * d;
        cA -= invMassA * P;
        aA -= invIA * Cross(rA_, P);
        cB += invMassB * P;
        aB += invIB * Cross(rB_, P);
        data.positions[indexA].c = cA;
        data.positions[indexA].a = aA;
        data.positions[indexB].c = cB;
        data.positions[indexB].a = aB;
        return Abs(C) < kLinearSlop;
    }

    void RevoluteInit(const SolverData& data) {                         // b2revolutejoint.d:319-439
        indexA = bodyA->islandIndex;
        indexB = bodyB->islandIndex;
        localCenterA = bodyA->sweep.localCenter;
        localCenterB = bodyB->sweep.localCenter;
        invMassA = bodyA->invMass;
        invMassB = bodyB->invMass;
        invIA = bodyA->invI;
        invIB = bodyB->invI;
        f32 aA = data.positions[indexA].a;
        Vec2 vA = data.velocities[indexA].v;
        f32 wA = data.velocities[indexA].w;
        f32 aB = data.positions[indexB].a;
        Vec2 vB = data.velocities[indexB].v;
        f32 wB = data.velocities[indexB].w;
        Rot qA(aA), qB(aB);
        rA = Mul(qA, localAnchorA - localCenterA);
        rB = Mul(qB, localAnchorB - localCenterB);
        f32 mA = invMassA, mB = invMassB;
        f32 iA = invIA, iB = invIB;
        bool fixedRotation = (iA + iB == 0.0f);
        massM.ex.x = ((mA + mB) + (rA.y * rA.y) * iA) + (rB.y * rB.y) * iB;
        massM.ey.x = (-rA.y * rA.x) * iA - (rB.y * rB.x) * iB;
        massM.ez.x = -rA.y * iA - rB.y * iB;
        massM.ex.y = massM.ey.x;
        massM.ey.y = ((mA + mB) + (rA.x * rA.x) * iA) + (rB.x * rB.x) * iB;
        massM.ez.y = rA.x * iA + rB.x * iB;
        massM.ex.z = massM.ez.x;
        massM.ey.z = massM.ez.y;
        massM.ez.z = iA + iB;
        motorMass = iA + iB;
        if (motorMass > 0.0f) motorMass = 1.0f / motorMass;
        if (enableMotor == false || fixedRotation) motorImpulse = 0.0f;
        if (enableLimit && fixedRotation == false) {
            f32 jointAngle = (aB - aA) - referenceAngle;
            if (Abs(upperAngle - lowerAngle) < 2.0f * kAngularSlop) {
                limitState = kEqualLimits;
            } else if (jointAngle <= lowerAngle) {
                if (limitState != kAtLowerLimit) impulse.z = 0.0f;
                limitState = kAtLowerLimit;
            } else if (jointAngle >= upperAngle) {
                if (limitState != kAtUpperLimit) impulse.z = 0.0f;
                limitState = kAtUpperLimit;
            } else {
                limitState = kInactiveLimit;
                impulse.z = 0.0f;
            }
        } else {
            limitState = kInactiveLimit;
        }
        if (data.step.warmStarting) {
            impulse *= data.step.dtRatio;
            motorImpulse *= data.step.dtRatio;
            Vec2 P(impulse.x, impulse.y);
            vA -= mA * P;
            wA -= iA * ((Cross(rA, P) + motorImpulse) + impulse.z);
            vB += mB * P;
            wB += iB * ((Cross(rB, P) + motorImpulse) + impulse.z);
        } else {
            impulse.SetZero();
            motorImpulse = 0.0f;
        }
        data.velocities[indexA].v = vA;
        data.velocities[indexA].w = wA;
        data.velocities[indexB].v = vB;
        data.velocities[indexB].w = wB;
    }

    void RevoluteSolveVelocity(const SolverData& data) {                // b2revolutejoint.d:441-549
        Vec2 vA = data.velocities[indexA].v;
        f32 wA = data.velocities[indexA].w;
        Vec2 vB = data.velocities[indexB].v;
        f32 wB = data.velocities[indexB].w;
        f32 mA = invMassA, mB = invMassB;
        f32 iA = invIA, iB = invIB;
        bool fixedRotation = (iA + iB == 0.0f);
        if (enableMotor && limitState != kEqualLimits && fixedRotation == false) {
            f32 Cdot = (wB - wA) - motorSpeed;
            f32 imp = -motorMass * Cdot;
            f32 oldImpulse = motorImpulse;
            f32 maxImpulse = data.step.dt * maxMotorTorque;
            motorImpulse = Clamp(motorImpulse + imp, -maxImpulse, maxImpulse);
            imp = motorImpulse - oldImpulse;
            wA -= iA * imp;
            wB += iB * imp;
        }
        if (enableLimit && limitState != kInactiveLimit && fixedRotation == false) {
            Vec2 Cdot1 = ((vB + Cross(wB, rB)) - vA) - Cross(wA, rA);
            f32 Cdot2 = wB - wA;
            Vec3 Cdot(Cdot1.x, Cdot1.y, Cdot2);
            Vec3 imp = -massM.Solve33(Cdot);
            if (limitState == kEqualLimits) {
                impulse += imp;
            } else if (limitState == kAtLowerLimit) {
                f32 newImpulse = impulse.z + imp.z;
                if (newImpulse < 0.0f) {
                    Vec2 rhs = -Cdot1 + impulse.z * Vec2(massM.ez.x, massM.ez.y);
                    Vec2 reduced = massM.Solve22(rhs);
                    imp.x = reduced.x;
                    imp.y = reduced.y;
                    imp.z = -impulse.z;
                    impulse.x += reduced.x;
                    impulse.y += reduced.y;
                    impulse.z = 0.0f;
                } else {
                    impulse += imp;
                }
            } else if (limitState == kAtUpperLimit) {
                f32 newImpulse = impulse.z + imp.z;
                if (newImpulse > 0.0f) {
                    Vec2 rhs = -Cdot1 + impulse.z * Vec2(massM.ez.x, massM.ez.y);
                    Vec2 reduced = massM.Solve22(rhs);
                    imp.x = reduced.x;
                    imp.y = reduced.y;
                    imp.z = -impulse.z;
                    impulse.x += reduced.x;
                    impulse.y += reduced.y;
                    impulse.z = 0.0f;
                } else {
                    impulse += imp;
                }
            }
            Vec2 P(imp.x, imp.y);
            vA -= mA * P;
            wA -= iA * (Cross(rA, P) + imp.z);
            vB += mB * P;
            wB += iB * (Cross(rB, P) + imp.z);
        } else {
            Vec2 Cdot = ((vB + Cross(wB, rB)) - vA) - Cross(wA, rA);
            Vec2 imp = massM.Solve22(-Cdot);
            impulse.x += imp.x;
            impulse.y += imp.y;
            vA -= mA * imp;
            wA -= iA * Cross(rA, imp);
            vB += mB * imp;
            wB += iB * Cross(rB, imp);
        }
        data.velocities[indexA].v = vA;
        data.velocities[indexA].w = wA;
        data.velocities[indexB].v = vB;
        data.velocities[indexB].w = wB;
    }

    bool RevoluteSolvePosition(const SolverData& data) {                // b2revolutejoint.d:551-636
        Vec2 cA = data.positions[indexA].c;
        f32 aA = data.positions[indexA].a;
        Vec2 cB = data.positions[indexB].c;
        f32 aB = data.positions[indexB].a;
        Rot qA(aA), qB(aB);
        f32 angularError = 0.0f;
        f32 positionError = 0.0f;
        bool fixedRotation = (invIA + invIB == 0.0f);
        if (enableLimit && limitState != kInactiveLimit && fixedRotation == false) {
            f32 angle = (aB - aA) - referenceAngle;
            f32 limitImpulse = 0.0f;
            if (limitState == kEqualLimits) {
                f32 C = Clamp(angle - lowerAngle, -kMaxAngularCorrection, kMaxAngularCorrection);
                limitImpulse = -motorMass * C;
                angularError = Abs(C);
            } else if (limitState == kAtLowerLimit) {
                f32 C = angle - lowerAngle;
                angularError = -C;
                C = Clamp(C + kAngularSlop, -kMaxAngularCorrection, 0.0f);
                limitImpulse = -motorMass * C;
            } else if (limitState == kAtUpperLimit) {
                f32 C = angle - upperAngle;
                angularError = C;
                C = Clamp(C - kAngularSlop, 0.0f, kMaxAngularCorrection);
                limitImpulse = -motorMass * C;
            }
            aA -= invIA * limitImpulse;
            aB += invIB * limitImpulse;
        }
        {
            qA.Set(aA);
            qB.Set(aB);
            Vec2 rA_ = Mul(qA, localAnchorA - localCenterA);
            Vec2 rB_ = Mul(qB, localAnchorB - localCenterB);
            Vec2 C = ((cB + rB_) - cA) - rA_;
            positionError = C.Length();
            f32 mA = invMassA, mB = invMassB;
            f32 iA = invIA, iB = invIB;
            Mat22 K;
            K.ex.x = ((mA + mB) + (iA * rA_.y) * rA_.y) + (iB * rB_.y) * rB_.y;
            K.ex.y = ((-iA * rA_.x) * rA_.y) - (iB * rB_.x) * rB_.y;
            K.ey.x = K.ex.y;
            K.ey.y = ((mA + mB) + (iA * rA_.x) * rA_.x) + (iB * rB_.x) * rB_.x;
            Vec2 imp = -K.Solve(C);
            cA -= mA * imp;
            aA -= iA * Cross(rA_, imp);
            cB += mB * imp;
            aB += iB * Cross(rB_, imp);
        }
        data.positions[indexA].c = cA;
        data.positions[indexA].a = aA;
        data.positions[indexB].c = cB;
        data.positions[indexB].a = aB;
        return positionError <= kLinearSlop && angularError <= kAngularSlop;
    }
};

bool Body::ShouldCollide(const Body* other) const {                     // b2body.d:1149-1170
    if (type != kDynamicBody && other->type != kDynamicBody) return false;
    for (JointEdge* jn = jointList; jn; jn = jn->next) {
        if (jn->other == other) {
            if (jn->joint->collideConnected == false) return false;
        }
    }
    return true;
}

// ------------------------------------------------------------ contact solver
// contacts/b2contactsolver.d
struct VelocityConstraintPoint { Vec2 rA, rB; f32 normalImpulse = 0, tangentImpulse = 0, normalMass = 0, tangentMass = 0, velocityBias = 0; };
struct ContactVelocityConstraint {
    VelocityConstraintPoint points[kMaxManifoldPoints];
    Vec2 normal;
    Mat22 normalMass;
    Mat22 K;
    int indexA = 0, indexB = 0;
    f32 invMassA = 0, invMassB = 0, invIA = 0, invIB = 0;
    f32 friction = 0, restitution = 0, tangentSpeed = 0;
    int pointCount = 0;
    int contactIndex = 0;
};
struct ContactPositionConstraint {
    Vec2 localPoints[kMaxManifoldPoints];
    Vec2 localNormal, localPoint;
    int indexA = 0, indexB = 0;
    f32 invMassA = 0, invMassB = 0;
    Vec2 localCenterA, localCenterB;
    f32 invIA = 0, invIB = 0;
    int type = 0;
    f32 radiusA = 0, radiusB = 0;
    int pointCount = 0;
};

struct PositionSolverManifold {                                         // b2contactsolver.d:816-851
    Vec2 normal, point;
    f32 separation = 0;
    void Initialize(const ContactPositionConstraint* pc, const Transform& xfA, const Transform& xfB, int index) {
        switch (pc->type) {
        case kManifoldCircles: {
            Vec2 pointA = Mul(xfA, pc->localPoint);
            Vec2 pointB = Mul(xfB, pc->localPoints[0]);
            normal = pointB - pointA;
            normal.Normalize();
            point = 0.5f * (pointA + pointB);
            separation = (Dot(pointB - pointA, normal) - pc->radiusA) - pc->radiusB;
        } break;
        case kManifoldFaceA: {
            normal = Mul(xfA.q, pc->localNormal);
            Vec2 planePoint = Mul(xfA, pc->localPoint);
            Vec2 clipPoint = Mul(xfB, pc->localPoints[index]);
            separation = (Dot(clipPoint - planePoint, normal) - pc->radiusA) - pc->radiusB;
            point = clipPoint;
        } break;
        case kManifoldFaceB: {
            normal = Mul(xfB.q, pc->localNormal);
            Vec2 planePoint = Mul(xfB, pc->localPoint);
            Vec2 clipPoint = Mul(xfA, pc->localPoints[index]);
            separation = (Dot(clipPoint - planePoint, normal) - pc->radiusA) - pc->radiusB;
            point = clipPoint;
            normal = -normal;
        } break;
        default: break;
        }
    }
};

struct ContactSolver {
    TimeStep step;
    Position* positions = nullptr;
    Velocity* velocities = nullptr;
    std::vector<ContactPositionConstraint> pcs;
    std::vector<ContactVelocityConstraint> vcs;
    Contact** contacts = nullptr;
    int count = 0;

    ContactSolver(const TimeStep& st, Contact** cs, int n, Position* pos, Velocity* vel) {  // :244-329
        step = st;
        count = n;
        pcs.resize(n);
        vcs.resize(n);
        positions = pos;
        velocities = vel;
        contacts = cs;
        for (int i = 0; i < count; ++i) {
            Contact* contact = contacts[i];
            Fixture* fixtureA = contact->fixtureA;
            Fixture* fixtureB = contact->fixtureB;
            f32 radiusA = fixtureA->shape.radius;
            f32 radiusB = fixtureB->shape.radius;
            Body* bodyA = fixtureA->body;
            Body* bodyB = fixtureB->body;
            Manifold* manifold = &contact->manifold;
            int pointCount = manifold->pointCount;
            ContactVelocityConstraint* vc = &vcs[i];
            vc->friction = contact->friction;
            vc->restitution = contact->restitution;
            vc->tangentSpeed = contact->tangentSpeed;
            vc->indexA = bodyA->islandIndex;
            vc->indexB = bodyB->islandIndex;
            vc->invMassA = bodyA->invMass;
            vc->invMassB = bodyB->invMass;
            vc->invIA = bodyA->invI;
            vc->invIB = bodyB->invI;
            vc->contactIndex = i;
            vc->pointCount = pointCount;
            vc->K.SetZero();
            vc->normalMass.SetZero();
            ContactPositionConstraint* pc = &pcs[i];
            pc->indexA = bodyA->islandIndex;
            pc->indexB = bodyB->islandIndex;
            pc->invMassA = bodyA->invMass;
            pc->invMassB = bodyB->invMass;
            pc->localCenterA = bodyA->sweep.localCenter;
            pc->localCenterB = bodyB->sweep.localCenter;
            pc->invIA = bodyA->invI;
            pc->invIB = bodyB->invI;
            pc->localNormal = manifold->localNormal;
            pc->localPoint = manifold->localPoint;
            pc->pointCount = pointCount;
            pc->radiusA = radiusA;
            pc->radiusB = radiusB;
            pc->type = manifold->type;
            for (int j = 0; j < pointCount; ++j) {
                ManifoldPoint* cp = manifold->points + j;
                VelocityConstraintPoint* vcp = vc->points + j;
                if (step.warmStarting) {
                    vcp->normalImpulse = step.dtRatio * cp->normalImpulse;
                    vcp->tangentImpulse = step.dtRatio * cp->tangentImpulse;
                } else {
                    vcp->normalImpulse = 0.0f;
                    vcp->tangentImpulse = 0.0f;
                }
                vcp->rA.SetZero();
                vcp->rB.SetZero();
                vcp->normalMass = 0.0f;
                vcp->tangentMass = 0.0f;
                vcp->velocityBias = 0.0f;
                pc->localPoints[j] = cp->localPoint;
            }
        }
    }

    void InitializeVelocityConstraints() {                              // :338-450
        for (int i = 0; i < count; ++i) {
            ContactVelocityConstraint* vc = &vcs[i];
            ContactPositionConstraint* pc = &pcs[i];
            f32 radiusA = pc->radiusA;
            f32 radiusB = pc->radiusB;
            Manifold* manifold = &contacts[vc->contactIndex]->manifold;
            int indexA = vc->indexA;
            int indexB = vc->indexB;
            f32 mA = vc->invMassA;
            f32 mB = vc->invMassB;
            f32 iA = vc->invIA;
            f32 iB = vc->invIB;
            Vec2 localCenterA = pc->localCenterA;
            Vec2 localCenterB = pc->localCenterB;
            Vec2 cA = positions[indexA].c;
            f32 aA = positions[indexA].a;
            Vec2 vA = velocities[indexA].v;
            f32 wA = velocities[indexA].w;
            Vec2 cB = positions[indexB].c;
            f32 aB = positions[indexB].a;
            Vec2 vB = velocities[indexB].v;
            f32 wB = velocities[indexB].w;
            Transform xfA, xfB;
            xfA.q.Set(aA);
            xfB.q.Set(aB);
            xfA.p = cA - Mul(xfA.q, localCenterA);
            xfB.p = cB - Mul(xfB.q, localCenterB);
            WorldManifold worldManifold;
            worldManifold.Initialize(manifold, xfA, radiusA, xfB, radiusB);
            vc->normal = worldManifold.normal;
            int pointCount = vc->pointCount;
            for (int j = 0; j < pointCount; ++j) {
                VelocityConstraintPoint* vcp = vc->points + j;
                vcp->rA = worldManifold.points[j] - cA;
                vcp->rB = worldManifold.points[j] - cB;
                f32 rnA = Cross(vcp->rA, vc->normal);
                f32 rnB = Cross(vcp->rB, vc->normal);
                f32 kNormal = ((mA + mB) + (iA * rnA) * rnA) + (iB * rnB) * rnB;
                vcp->normalMass = kNormal > 0.0f ? 1.0f / kNormal : 0.0f;
                Vec2 tangent = Cross(vc->normal, 1.0f);
                f32 rtA = Cross(vcp->rA, tangent);
                f32 rtB = Cross(vcp->rB, tangent);
                f32 kTangent = ((mA + mB) + (iA * rtA) * rtA) + (iB * rtB) * rtB;
                vcp->tangentMass = kTangent > 0.0f ? 1.0f / kTangent : 0.0f;
                vcp->velocityBias = 0.0f;
                f32 vRel = Dot(vc->normal, ((vB + Cross(wB, vcp->rB)) - vA) - Cross(wA, vcp->rA));
                if (vRel < -kVelocityThreshold) vcp->velocityBias = -vc->restitution * vRel;
            }
            if (vc->pointCount == 2) {
                VelocityConstraintPoint* vcp1 = vc->points + 0;
                VelocityConstraintPoint* vcp2 = vc->points + 1;
                f32 rn1A = Cross(vcp1->rA, vc->normal);
                f32 rn1B = Cross(vcp1->rB, vc->normal);
                f32 rn2A = Cross(vcp2->rA, vc->normal);
                f32 rn2B = Cross(vcp2->rB, vc->normal);
                f32 k11 = ((mA + mB) + (iA * rn1A) * rn1A) + (iB * rn1B) * rn1B;
                f32 k22 = ((mA + mB) + (iA * rn2A) * rn2A) + (iB * rn2B) * rn2B;
                f32 k12 = ((mA + mB) + (iA * rn1A) * rn2A) + (iB * rn1B) * rn2B;
                const f32 k_maxConditionNumber = 1000.0f;
                if (k11 * k11 < k_maxConditionNumber * (k11 * k22 - k12 * k12)) {
                    vc->K.ex.Set(k11, k12);
                    vc->K.ey.Set(k12, k22);
                    vc->normalMass = vc->K.GetInverse();
                } else {
                    vc->pointCount = 1;
                }
            }
        }
    }

    void WarmStart() {                                                  // :452-490
        for (int i = 0; i < count; ++i) {
            ContactVelocityConstraint* vc = &vcs[i];
            int indexA = vc->indexA;
            int indexB = vc->indexB;
            f32 mA = vc->invMassA;
            f32 iA = vc->invIA;
            f32 mB = vc->invMassB;
            f32 iB = vc->invIB;
            int pointCount = vc->pointCount;
            Vec2 vA = velocities[indexA].v;
            f32 wA = velocities[indexA].w;
            Vec2 vB = velocities[indexB].v;
            f32 wB = velocities[indexB].w;
            Vec2 normal = vc->normal;
            Vec2 tangent = Cross(normal, 1.0f);
            for (int j = 0; j < pointCount; ++j) {
                VelocityConstraintPoint* vcp = vc->points + j;
                Vec2 P = vcp->normalImpulse * normal + vcp->tangentImpulse * tangent;
                wA -= iA * Cross(vcp->rA, P);
                vA -= mA * P;
                wB += iB * Cross(vcp->rB, P);
                vB += mB * P;
            }
            velocities[indexA].v = vA;
            velocities[indexA].w = wA;
            velocities[indexB].v = vB;
            velocities[indexB].w = wB;
        }
    }

    void SolveVelocityConstraints() {                                   // :492-772
        for (int i = 0; i < count; ++i) {
            ContactVelocityConstraint* vc = &vcs[i];
            int indexA = vc->indexA;
            int indexB = vc->indexB;
            f32 mA = vc->invMassA;
            f32 iA = vc->invIA;
            f32 mB = vc->invMassB;
            f32 iB = vc->invIB;
            int pointCount = vc->pointCount;
            Vec2 vA = velocities[indexA].v;
            f32 wA = velocities[indexA].w;
            Vec2 vB = velocities[indexB].v;
            f32 wB = velocities[indexB].w;
            Vec2 normal = vc->normal;
            Vec2 tangent = Cross(normal, 1.0f);
            f32 friction = vc->friction;
            for (int j = 0; j < pointCount; ++j) {
                VelocityConstraintPoint* vcp = vc->points + j;
                Vec2 dv = ((vB + Cross(wB, vcp->rB)) - vA) - Cross(wA, vcp->rA);
                f32 vt = Dot(dv, tangent) - vc->tangentSpeed;
                f32 lambda = vcp->tangentMass * (-vt);
                f32 maxFriction = friction * vcp->normalImpulse;
                f32 newImpulse = Clamp(vcp->tangentImpulse + lambda, -maxFriction, maxFriction);
                lambda = newImpulse - vcp->tangentImpulse;
                vcp->tangentImpulse = newImpulse;
                Vec2 P = lambda * tangent;
                vA -= mA * P;
                wA -= iA * Cross(vcp->rA, P);
                vB += mB * P;
                wB += iB * Cross(vcp->rB, P);
            }
            if (pointCount == 1) {
                for (int idx = 0; idx < pointCount; ++idx) {
                    VelocityConstraintPoint* vcp = vc->points + idx;
                    Vec2 dv = ((vB + Cross(wB, vcp->rB)) - vA) - Cross(wA, vcp->rA);
                    f32 vn = Dot(dv, normal);
                    f32 lambda = -vcp->normalMass * (vn - vcp->velocityBias);
                    f32 newImpulse = Max(vcp->normalImpulse + lambda, 0.0f);
                    lambda = newImpulse - vcp->normalImpulse;
                    vcp->normalImpulse = newImpulse;
                    Vec2 P = lambda * normal;
                    vA -= mA * P;
                    wA -= iA * Cross(vcp->rA, P);
                    vB += mB * P;
                    wB += iB * Cross(vcp->rB, P);
                }
            } else {
                VelocityConstraintPoint* cp1 = vc->points + 0;
                VelocityConstraintPoint* cp2 = vc->points + 1;
                Vec2 a(cp1->normalImpulse, cp2->normalImpulse);
                Vec2 dv1 = ((vB + Cross(wB, cp1->rB)) - vA) - Cross(wA, cp1->rA);
                Vec2 dv2 = ((vB + Cross(wB, cp2->rB)) - vA) - Cross(wA, cp2->rA);
                f32 vn1 = Dot(dv1, normal);
                f32 vn2 = Dot(dv2, normal);
                Vec2 b;
                b.x = vn1 - cp1->velocityBias;
                b.y = vn2 - cp2->velocityBias;
                b -= Mul(vc->K, a);
                for (;;) {
                    Vec2 x = -Mul(vc->normalMass, b);
                    if (x.x >= 0.0f && x.y >= 0.0f) {
                        Vec2 d = x - a;
                        Vec2 P1 = d.x * normal;
                        Vec2 P2 = d.y * normal;
                        vA -= mA * (P1 + P2);
                        wA -= iA * (Cross(cp1->rA, P1) + Cross(cp2->rA, P2));
                        vB += mB * (P1 + P2);
                        wB += iB * (Cross(cp1->rB, P1) + Cross(cp2->rB, P2));
                        cp1->normalImpulse = x.x;
                        cp2->normalImpulse = x.y;
                        break;
                    }
                    x.x = -cp1->normalMass * b.x;
                    x.y = 0.0f;
                    vn1 = 0.0f;
                    vn2 = vc->K.ex.y * x.x + b.y;
                    if (x.x >= 0.0f && vn2 >= 0.0f) {
                        Vec2 d = x - a;
                        Vec2 P1 = d.x * normal;
                        Vec2 P2 = d.y * normal;
                        vA -= mA * (P1 + P2);
                        wA -= iA * (Cross(cp1->rA, P1) + Cross(cp2->rA, P2));
                        vB += mB * (P1 + P2);
                        wB += iB * (Cross(cp1->rB, P1) + Cross(cp2->rB, P2));
                        cp1->normalImpulse = x.x;
                        cp2->normalImpulse = x.y;
                        break;
                    }
                    x.x = 0.0f;
                    x.y = -cp2->normalMass * b.y;
                    vn1 = vc->K.ey.x * x.y + b.x;
                    vn2 = 0.0f;
                    if (x.y >= 0.0f && vn1 >= 0.0f) {
                        Vec2 d = x - a;
                        Vec2 P1 = d.x * normal;
                        Vec2 P2 = d.y * normal;
                        vA -= mA * (P1 + P2);
                        wA -= iA * (Cross(cp1->rA, P1) + Cross(cp2->rA, P2));
                        vB += mB * (P1 + P2);
                        wB += iB * (Cross(cp1->rB, P1) + Cross(cp2->rB, P2));
                        cp1->normalImpulse = x.x;
                        cp2->normalImpulse = x.y;
                        break;
                    }
                    x.x = 0.0f;
                    x.y = 0.0f;
                    vn1 = b.x;
                    vn2 = b.y;
                    if (vn1 >= 0.0f && vn2 >= 0.0f) {
                        Vec2 d = x - a;
                        Vec2 P1 = d.x * normal;
                        Vec2 P2 = d.y * normal;
                        vA -= mA * (P1 + P2);
                        wA -= iA * (Cross(cp1->rA, P1) + Cross(cp2->rA, P2));
                        vB += mB * (P1 + P2);
                        wB += iB * (Cross(cp1->rB, P1) + Cross(cp2->rB, P2));
                        cp1->normalImpulse = x.x;
                        cp2->normalImpulse = x.y;
                        break;
                    }
                    break;
                }
            }
            velocities[indexA].v = vA;
            velocities[indexA].w = wA;
            velocities[indexB].v = vB;
            velocities[indexB].w = wB;
        }
    }

    void StoreImpulses() {                                              // :774-787
        for (int i = 0; i < count; ++i) {
            ContactVelocityConstraint* vc = &vcs[i];
            Manifold* manifold = &contacts[vc->contactIndex]->manifold;
            for (int j = 0; j < vc->pointCount; ++j) {
                manifold->points[j].normalImpulse = vc->points[j].normalImpulse;
                manifold->points[j].tangentImpulse = vc->points[j].tangentImpulse;
            }
        }
    }

    bool SolvePositionConstraintsImpl(bool toi, int toiIndexA, int toiIndexB) {  // :73-242
        f32 minSeparation = 0.0f;
        for (int i = 0; i < count; ++i) {
            ContactPositionConstraint* pc = &pcs[i];
            int indexA = pc->indexA;
            int indexB = pc->indexB;
            Vec2 localCenterA = pc->localCenterA;
            Vec2 localCenterB = pc->localCenterB;
            int pointCount = pc->pointCount;
            f32 mA, iA, mB, iB;
            if (!toi) {
                mA = pc->invMassA; iA = pc->invIA; mB = pc->invMassB; iB = pc->invIB;
            } else {
                mA = 0.0f; iA = 0.0f;
                if (indexA == toiIndexA || indexA == toiIndexB) { mA = pc->invMassA; iA = pc->invIA; }
                mB = 0.0f; iB = 0.0f;
                if (indexB == toiIndexA || indexB == toiIndexB) { mB = pc->invMassB; iB = pc->invIB; }
            }
            Vec2 cA = positions[indexA].c;
            f32 aA = positions[indexA].a;
            Vec2 cB = positions[indexB].c;
            f32 aB = positions[indexB].a;
            for (int j = 0; j < pointCount; ++j) {
                Transform xfA, xfB;
                xfA.q.Set(aA);
                xfB.q.Set(aB);
                xfA.p = cA - Mul(xfA.q, localCenterA);
                xfB.p = cB - Mul(xfB.q, localCenterB);
                PositionSolverManifold psm;
                psm.Initialize(pc, xfA, xfB, j);
                Vec2 normal = psm.normal;
                Vec2 point = psm.point;
                f32 separation = psm.separation;
                Vec2 rA = point - cA;
                Vec2 rB = point - cB;
                minSeparation = Min(minSeparation, separation);
                f32 C = Clamp((toi ? kToiBaumgarte : kBaumgarte) * (separation + kLinearSlop),
                              -kMaxLinearCorrection, 0.0f);
                f32 rnA = Cross(rA, normal);
                f32 rnB = Cross(rB, normal);
                f32 K = ((mA + mB) + (iA * rnA) * rnA) + (iB * rnB) * rnB;
                f32 impulse = K > 0.0f ? -C / K : 0.0f;
                Vec2 P = impulse * normal;
                cA -= mA * P;
                aA -= iA * Cross(rA, P);
                cB += mB * P;
                aB += iB * Cross(rB, P);
            }
            positions[indexA].c = cA;
            positions[indexA].a = aA;
            positions[indexB].c = cB;
            positions[indexB].a = aB;
        }
        return toi ? minSeparation >= -1.5f * kLinearSlop : minSeparation >= -3.0f * kLinearSlop;
    }
};

// ------------------------------------------------------------ island
struct Profile { };

struct Island {                                                         // dynamics/b2island.d
    std::vector<Body*> bodies;
    std::vector<Contact*> contacts;
    std::vector<Joint*> joints;
    std::vector<Position> positions;
    std::vector<Velocity> velocities;
    Listener* listener = nullptr;
    int bodyCapacity = 0, contactCapacity = 0;

    void Clear() { bodies.clear(); contacts.clear(); joints.clear(); }
    void Add(Body* b) { b->islandIndex = (int)bodies.size(); bodies.push_back(b); }
    void Add(Contact* c) { contacts.push_back(c); }
    void Add(Joint* j) { joints.push_back(j); }

    void Report(const std::vector<ContactVelocityConstraint>& constraints) {  // b2island.d:438-462
        if (!listener) return;
        for (size_t i = 0; i < contacts.size(); ++i) {
            const ContactVelocityConstraint* vc = &constraints[i];
            f32 ni[2] = {0, 0}, ti[2] = {0, 0};
            for (int j = 0; j < vc->pointCount; ++j) {
                ni[j] = vc->points[j].normalImpulse;
                ti[j] = vc->points[j].tangentImpulse;
            }
            listener->PostSolve(contacts[i], vc->pointCount, ni, ti);
        }
    }

    void Solve(const TimeStep& step, Vec2 gravity, bool allowSleep) {   // b2island.d:75-280
        f32 h = step.dt;
        int bodyCount = (int)bodies.size();
        positions.assign(bodyCount, Position());
        velocities.assign(bodyCount, Velocity());
        for (int i = 0; i < bodyCount; ++i) {
            Body* b = bodies[i];
            Vec2 c = b->sweep.c;
            f32 a = b->sweep.a;
            Vec2 v = b->linearVelocity;
            f32 w = b->angularVelocity;
            b->sweep.c0 = b->sweep.c;
            b->sweep.a0 = b->sweep.a;
            if (b->type == kDynamicBody) {
                v += h * (b->gravityScale * gravity + b->invMass * b->force);
                w += (h * b->invI) * b->torque;
                v *= 1.0f / (1.0f + h * b->linearDamping);
                w *= 1.0f / (1.0f + h * b->angularDamping);
            }
            positions[i].c = c;
            positions[i].a = a;
            velocities[i].v = v;
            velocities[i].w = w;
        }
        SolverData solverData;
        solverData.step = step;
        solverData.positions = positions.data();
        solverData.velocities = velocities.data();
        ContactSolver contactSolver(step, contacts.data(), (int)contacts.size(), positions.data(), velocities.data());
        contactSolver.InitializeVelocityConstraints();
        if (step.warmStarting) contactSolver.WarmStart();
        for (Joint* j : joints) j->InitVelocityConstraints(solverData);
        for (int i = 0; i < step.velocityIterations; ++i) {
            for (Joint* j : joints) j->SolveVelocityConstraints(solverData);
            contactSolver.SolveVelocityConstraints();
        }
        contactSolver.StoreImpulses();
        for (int i = 0; i < bodyCount; ++i) {
            Vec2 c = positions[i].c;
            f32 a = positions[i].a;
            Vec2 v = velocities[i].v;
            f32 w = velocities[i].w;
            Vec2 translation = h * v;
            if (Dot(translation, translation) > kMaxTranslationSquared) {
                f32 ratio = kMaxTranslation / translation.Length();
                v *= ratio;
            }
            f32 rotation = h * w;
            if (rotation * rotation > kMaxRotationSquared) {
                f32 ratio = kMaxRotation / Abs(rotation);
                w *= ratio;
            }
            c += h * v;
            a += h * w;
            positions[i].c = c;
            positions[i].a = a;
            velocities[i].v = v;
            velocities[i].w = w;
        }
        bool positionSolved = false;
        for (int i = 0; i < step.positionIterations; ++i) {
            bool contactsOkay = contactSolver.SolvePositionConstraintsImpl(false, 0, 0);
            bool jointsOkay = true;
            for (Joint* j : joints) {
                bool jointOkay = j->SolvePositionConstraints(solverData);
                jointsOkay = jointsOkay && jointOkay;
            }
            if (contactsOkay && jointsOkay) { positionSolved = true; break; }
        }
        for (int i = 0; i < bodyCount; ++i) {
            Body* body = bodies[i];
            body->sweep.c = positions[i].c;
            body->sweep.a = positions[i].a;
            body->linearVelocity = velocities[i].v;
            body->angularVelocity = velocities[i].w;
            body->SynchronizeTransform();
        }
        Report(contactSolver.vcs);
        if (allowSleep) {
            f32 minSleepTime = kMaxFloat;
            const f32 linTolSqr = kLinearSleepTolerance * kLinearSleepTolerance;
            const f32 angTolSqr = kAngularSleepTolerance * kAngularSleepTolerance;
            for (int i = 0; i < bodyCount; ++i) {
                Body* b = bodies[i];
                if (b->type == kStaticBody) continue;
                if ((b->flags & kBodyAutoSleep) == 0 || b->angularVelocity * b->angularVelocity > angTolSqr ||
                    Dot(b->linearVelocity, b->linearVelocity) > linTolSqr) {
                    b->sleepTime = 0.0f;
                    minSleepTime = 0.0f;
                } else {
                    b->sleepTime += h;
                    minSleepTime = Min(minSleepTime, b->sleepTime);
                }
            }
            if (minSleepTime >= kTimeToSleep && positionSolved) {
                for (int i = 0; i < bodyCount; ++i) bodies[i]->SetAwake(false);
            }
        }
    }

    void SolveTOI(const TimeStep& subStep, int toiIndexA, int toiIndexB) {  // b2island.d:282-416
        int bodyCount = (int)bodies.size();
        positions.assign(bodyCount, Position());
        velocities.assign(bodyCount, Velocity());
        for (int i = 0; i < bodyCount; ++i) {
            Body* b = bodies[i];
            positions[i].c = b->sweep.c;
            positions[i].a = b->sweep.a;
            velocities[i].v = b->linearVelocity;
            velocities[i].w = b->angularVelocity;
        }
        ContactSolver contactSolver(subStep, contacts.data(), (int)contacts.size(), positions.data(), velocities.data());
        for (int i = 0; i < subStep.positionIterations; ++i) {
            bool contactsOkay = contactSolver.SolvePositionConstraintsImpl(true, toiIndexA, toiIndexB);
            if (contactsOkay) break;
        }
        bodies[toiIndexA]->sweep.c0 = positions[toiIndexA].c;
        bodies[toiIndexA]->sweep.a0 = positions[toiIndexA].a;
        bodies[toiIndexB]->sweep.c0 = positions[toiIndexB].c;
        bodies[toiIndexB]->sweep.a0 = positions[toiIndexB].a;
        contactSolver.InitializeVelocityConstraints();
        for (int i = 0; i < subStep.velocityIterations; ++i) contactSolver.SolveVelocityConstraints();
        f32 h = subStep.dt;
        for (int i = 0; i < bodyCount; ++i) {
            Vec2 c = positions[i].c;
            f32 a = positions[i].a;
            Vec2 v = velocities[i].v;
            f32 w = velocities[i].w;
            Vec2 translation = h * v;
            if (Dot(translation, translation) > kMaxTranslationSquared) {
                f32 ratio = kMaxTranslation / translation.Length();
                v *= ratio;
            }
            f32 rotation = h * w;
            if (rotation * rotation > kMaxRotationSquared) {
                f32 ratio = kMaxRotation / Abs(rotation);
                w *= ratio;
            }
            c += h * v;
            a += h * w;
            positions[i].c = c;
            positions[i].a = a;
            velocities[i].v = v;
            velocities[i].w = w;
            Body* body = bodies[i];
            body->sweep.c = c;
            body->sweep.a = a;
            body->linearVelocity = v;
            body->angularVelocity = w;
            body->SynchronizeTransform();
        }
        Report(contactSolver.vcs);
    }
};

// ------------------------------------------------------------ broadphase + contact manager
struct Pair { int proxyIdA, proxyIdB; };

struct ContactManager;

struct BroadPhase {                                                     // collision/b2broadphase.d
    DynamicTree tree;
    int proxyCount = 0;
    std::vector<int> moveBuffer;
    std::vector<Pair> pairBuffer;
    int queryProxyId = -1;

    int CreateProxy(const AABB& aabb, void* userData) {
        int proxyId = tree.CreateProxy(aabb, userData);
        ++proxyCount;
        BufferMove(proxyId);
        return proxyId;
    }
    void MoveProxy(int proxyId, const AABB& aabb, Vec2 displacement) {
        bool buffer = tree.MoveProxy(proxyId, aabb, displacement);
        if (buffer) BufferMove(proxyId);
    }
    void BufferMove(int proxyId) { moveBuffer.push_back(proxyId); }
    void DestroyProxy(int proxyId) {                                    // b2broadphase.d: DestroyProxy, UnBufferMove
        for (int& id : moveBuffer)
            if (id == proxyId) id = -1;
        --proxyCount;
        tree.DestroyProxy(proxyId);
    }
    bool TestOverlapProxies(int a, int b) const { return TestOverlap(tree.nodes[a].aabb, tree.nodes[b].aabb); }
    bool QueryCallback(int proxyId) {                                   // b2broadphase.d:271-294
        if (proxyId == queryProxyId) return true;
        Pair p;
        p.proxyIdA = Min(proxyId, queryProxyId);
        p.proxyIdB = Max(proxyId, queryProxyId);
        pairBuffer.push_back(p);
        return true;
    }
    void UpdatePairs(ContactManager* cm);                               // b2broadphase.d:139-195
};

static bool FilterShouldCollide(const Fixture* fixtureA, const Fixture* fixtureB);

// b2ContactFilter (b2worldcallbacks.d:47-64): the default rule, which a user subclass overrides
struct ContactFilter {
    virtual ~ContactFilter() {}
    virtual bool ShouldCollide(Fixture* a, Fixture* b) { return FilterShouldCollide(a, b); }
};

// A user's b2ContactFilter: fixtures of classes a and b collide when bit b of row a is set,
// optionally together with the default rule (a subclass calling the base class first)
struct TableFilter : ContactFilter {
    uint64_t table[64] = {};
    bool withDefault = true;
    bool ShouldCollide(Fixture* a, Fixture* b) override {
        const bool t = ((table[a->fclass & 63] >> (b->fclass & 63)) & 1u) != 0;
        return withDefault ? (ContactFilter::ShouldCollide(a, b) && t) : t;
    }
};

struct ContactManager {                                                 // dynamics/b2contactmanager.d
    BroadPhase broadPhase;
    Contact* contactList = nullptr;
    int contactCount = 0;
    Listener* listener = nullptr;
    ContactFilter defaultFilter;                                        // b2_defaultFilter
    ContactFilter* filter = &defaultFilter;                              // b2World.SetContactFilter

    void AddPair(void* proxyUserDataA, void* proxyUserDataB);
    void FindNewContacts() { broadPhase.UpdatePairs(this); }
    void Destroy(Contact* c);
    void Collide();
};

static bool FilterShouldCollide(const Fixture* fixtureA, const Fixture* fixtureB) {  // b2worldcallbacks.d:52-64
    const Filter& filterA = fixtureA->filter;
    const Filter& filterB = fixtureB->filter;
    if (filterA.groupIndex == filterB.groupIndex && filterA.groupIndex != 0) return filterA.groupIndex > 0;
    bool collide = (filterA.maskBits & filterB.categoryBits) != 0 && (filterA.categoryBits & filterB.maskBits) != 0;
    return collide;
}

void BroadPhase::UpdatePairs(ContactManager* cm) {
    pairBuffer.clear();
    for (size_t i = 0; i < moveBuffer.size(); ++i) {
        queryProxyId = moveBuffer[i];
        if (queryProxyId == -1) continue;
        AABB fatAABB = tree.nodes[queryProxyId].aabb;
        tree.Query(this, fatAABB);
    }
    moveBuffer.clear();
    std::sort(pairBuffer.begin(), pairBuffer.end(), [](const Pair& p1, const Pair& p2) {
        if (p1.proxyIdA < p2.proxyIdA) return true;
        if (p1.proxyIdA == p2.proxyIdA) return p1.proxyIdB < p2.proxyIdB;
        return false;
    });
    size_t i = 0;
    while (i < pairBuffer.size()) {
        Pair primary = pairBuffer[i];
        void* userDataA = tree.nodes[primary.proxyIdA].userData;
        void* userDataB = tree.nodes[primary.proxyIdB].userData;
        cm->AddPair(userDataA, userDataB);
        ++i;
        while (i < pairBuffer.size()) {
            const Pair& pair = pairBuffer[i];
            if (pair.proxyIdA != primary.proxyIdA || pair.proxyIdB != primary.proxyIdB) break;
            ++i;
        }
    }
}

// b2contactmanager.d:52-176 (AddPair) with the registry of b2contact.d:358-439
void ContactManager::AddPair(void* proxyUserDataA, void* proxyUserDataB) {
    FixtureProxy* proxyA = (FixtureProxy*)proxyUserDataA;
    FixtureProxy* proxyB = (FixtureProxy*)proxyUserDataB;
    Fixture* fixtureA = proxyA->fixture;
    Fixture* fixtureB = proxyB->fixture;
    int indexA = proxyA->childIndex;
    int indexB = proxyB->childIndex;
    Body* bodyA = fixtureA->body;
    Body* bodyB = fixtureB->body;
    if (bodyA == bodyB) return;
    for (ContactEdge* edge = bodyB->contactList; edge; edge = edge->next) {
        if (edge->other == bodyA) {
            Fixture* fA = edge->contact->fixtureA;
            Fixture* fB = edge->contact->fixtureB;
            int iA = edge->contact->indexA;
            int iB = edge->contact->indexB;
            if (fA == fixtureA && fB == fixtureB && iA == indexA && iB == indexB) return;
            if (fA == fixtureB && fB == fixtureA && iA == indexB && iB == indexA) return;
        }
    }
    if (bodyB->ShouldCollide(bodyA) == false) return;
    if (filter->ShouldCollide(fixtureA, fixtureB) == false) return;
    // Contact.Create: the registry's primary order is (circle, circle), (polygon, circle),
    // (polygon, polygon), (edge, circle), (edge, polygon); edges do not collide with edges
    int type1 = fixtureA->shape.type;
    int type2 = fixtureB->shape.type;
    if (!((type1 == kCircle || type1 == kPolygon || type1 == kEdge) && (type2 == kCircle || type2 == kPolygon || type2 == kEdge)))
        return;
    if (type1 == kEdge && type2 == kEdge) return;
    Contact* c = new Contact();
    if ((type1 == kCircle && type2 == kPolygon) || (type1 != kEdge && type2 == kEdge)) {
        c->fixtureA = fixtureB; c->indexA = indexB;
        c->fixtureB = fixtureA; c->indexB = indexA;
    } else {
        c->fixtureA = fixtureA; c->indexA = indexA;
        c->fixtureB = fixtureB; c->indexB = indexB;
    }
    c->flags = kContactEnabled;                                         // b2contact.d:208-239
    c->manifold.pointCount = 0;
    c->toiCount = 0;
    c->friction = MixFriction(c->fixtureA->friction, c->fixtureB->friction);
    c->restitution = MixRestitution(c->fixtureA->restitution, c->fixtureB->restitution);
    c->tangentSpeed = 0.0f;
    fixtureA = c->fixtureA;
    fixtureB = c->fixtureB;
    bodyA = fixtureA->body;
    bodyB = fixtureB->body;
    c->prev = nullptr;
    c->next = contactList;
    if (contactList) contactList->prev = c;
    contactList = c;
    c->nodeA.contact = c;
    c->nodeA.other = bodyB;
    c->nodeA.prev = nullptr;
    c->nodeA.next = bodyA->contactList;
    if (bodyA->contactList) bodyA->contactList->prev = &c->nodeA;
    bodyA->contactList = &c->nodeA;
    c->nodeB.contact = c;
    c->nodeB.other = bodyA;
    c->nodeB.prev = nullptr;
    c->nodeB.next = bodyB->contactList;
    if (bodyB->contactList) bodyB->contactList->prev = &c->nodeB;
    bodyB->contactList = &c->nodeB;
    if (fixtureA->isSensor == false && fixtureB->isSensor == false) {
        bodyA->SetAwake(true);
        bodyB->SetAwake(true);
    }
    ++contactCount;
}

void ContactManager::Destroy(Contact* c) {                              // b2contactmanager.d:183-246
    Fixture* fixtureA = c->fixtureA;
    Fixture* fixtureB = c->fixtureB;
    Body* bodyA = fixtureA->body;
    Body* bodyB = fixtureB->body;
    if (listener && c->IsTouching()) listener->EndContact(c);
    if (c->prev) c->prev->next = c->next;
    if (c->next) c->next->prev = c->prev;
    if (c == contactList) contactList = c->next;
    if (c->nodeA.prev) c->nodeA.prev->next = c->nodeA.next;
    if (c->nodeA.next) c->nodeA.next->prev = c->nodeA.prev;
    if (&c->nodeA == bodyA->contactList) bodyA->contactList = c->nodeA.next;
    if (c->nodeB.prev) c->nodeB.prev->next = c->nodeB.next;
    if (c->nodeB.next) c->nodeB.next->prev = c->nodeB.prev;
    if (&c->nodeB == bodyB->contactList) bodyB->contactList = c->nodeB.next;
    // b2Contact.Destroy (b2contact.d:402-422)
    if (c->manifold.pointCount > 0 && fixtureA->isSensor == false && fixtureB->isSensor == false) {
        fixtureA->body->SetAwake(true);
        fixtureB->body->SetAwake(true);
    }
    delete c;
    --contactCount;
}

void ContactManager::Collide() {                                        // b2contactmanager.d:251-317
    Contact* c = contactList;
    while (c) {
        Fixture* fixtureA = c->fixtureA;
        Fixture* fixtureB = c->fixtureB;
        Body* bodyA = fixtureA->body;
        Body* bodyB = fixtureB->body;
        if (c->flags & kContactFilter) {
            if (bodyB->ShouldCollide(bodyA) == false) {
                Contact* cNuke = c; c = cNuke->next; Destroy(cNuke); continue;
            }
            if (filter->ShouldCollide(fixtureA, fixtureB) == false) {
                Contact* cNuke = c; c = cNuke->next; Destroy(cNuke); continue;
            }
            c->flags &= ~kContactFilter;
        }
        bool activeA = bodyA->IsAwake() && bodyA->type != kStaticBody;
        bool activeB = bodyB->IsAwake() && bodyB->type != kStaticBody;
        if (activeA == false && activeB == false) { c = c->next; continue; }
        int proxyIdA = fixtureA->proxy.proxyId;
        int proxyIdB = fixtureB->proxy.proxyId;
        bool overlap = broadPhase.TestOverlapProxies(proxyIdA, proxyIdB);
        if (overlap == false) {
            Contact* cNuke = c; c = cNuke->next; Destroy(cNuke); continue;
        }
        c->Update(listener);
        c = c->next;
    }
}


// ------------------------------------------------------------ world
// A b2ChainShape as created (b2chainshape.d:45-110): its vertex list (a loop repeats the first
// vertex), ghost vertices and the fixture data; its child edges are fixtures [first, first + count - 1).
struct ChainRec {
    std::vector<Vec2> vertices;
    Vec2 prevVertex, nextVertex;
    bool hasPrevVertex = false, hasNextVertex = false;
    f32 density = 0;
    int first = -1;
};

struct World {                                                          // dynamics/b2world.d
    enum { kNewFixture = 0x0001, kLocked = 0x0002, kClearForces = 0x0004 };
    std::vector<ChainRec> chains;
    Body* bodyList = nullptr;
    Joint* jointList = nullptr;
    int bodyCount = 0, jointCount = 0;
    Vec2 gravity;
    bool allowSleep = true;
    ContactManager contactManager;
    bool warmStarting = true, continuousPhysics = true, subStepping = false;
    bool stepComplete = true;
    uint32_t flags = kClearForces;
    f32 inv_dt0 = 0.0f;
    std::vector<Body*> bodiesByIndex;
    std::vector<Fixture*> fixturesByIndex;
    std::vector<Joint*> jointsByIndex;
    Listener recorder;
    bool recording = false;
    int lastToiEvents = 0, lastIslands = 0;

    ~World() {
        for (Contact* c = contactManager.contactList; c;) { Contact* n = c->next; delete c; c = n; }
        for (Body* b : bodiesByIndex) delete b;
        for (Fixture* f : fixturesByIndex) delete f;
        for (Joint* j : jointsByIndex) delete j;
    }

    Body* CreateBody(const dbox_body_def* bd) {                         // b2world.d:75-99, b2body.d:1030-1115
        Body* b = new Body();
        b->flags = 0;
        if (bd->bullet) b->flags |= kBodyBullet;
        if (bd->fixed_rotation) b->flags |= kBodyFixedRotation;
        if (bd->allow_sleep) b->flags |= kBodyAutoSleep;
        if (bd->awake) b->flags |= kBodyAwake;
        if (bd->active) b->flags |= kBodyActive;
        b->world = this;
        b->xf.p = Vec2(bd->position.x, bd->position.y);
        b->xf.q.Set(bd->angle);
        b->sweep.localCenter.SetZero();
        b->sweep.c0 = b->xf.p;
        b->sweep.c = b->xf.p;
        b->sweep.a0 = bd->angle;
        b->sweep.a = bd->angle;
        b->sweep.alpha0 = 0.0f;
        b->linearVelocity = Vec2(bd->linear_velocity.x, bd->linear_velocity.y);
        b->angularVelocity = bd->angular_velocity;
        b->linearDamping = bd->linear_damping;
        b->angularDamping = bd->angular_damping;
        b->gravityScale = bd->gravity_scale;
        b->force.SetZero();
        b->torque = 0.0f;
        b->sleepTime = 0.0f;
        b->type = bd->type;
        if (b->type == kDynamicBody) { b->mass = 1.0f; b->invMass = 1.0f; }
        else { b->mass = 0.0f; b->invMass = 0.0f; }
        b->I = 0.0f;
        b->invI = 0.0f;
        b->prev = nullptr;
        b->next = bodyList;
        if (bodyList) bodyList->prev = b;
        bodyList = b;
        ++bodyCount;
        b->index = (int)bodiesByIndex.size();
        bodiesByIndex.push_back(b);
        return b;
    }

    Fixture* CreateFixture(Body* body, const Shape& shape, const dbox_fixture_def* def) {  // b2body.d:116-155
        Fixture* f = new Fixture();
        f->friction = def->friction;
        f->restitution = def->restitution;
        f->body = body;
        f->next = nullptr;
        f->filter.categoryBits = def->category_bits;
        f->filter.maskBits = def->mask_bits;
        f->filter.groupIndex = def->group_index;
        f->isSensor = def->is_sensor != 0;
        f->shape = shape;
        f->proxy.fixture = nullptr;
        f->proxy.proxyId = -1;
        f->proxyCount = 0;
        f->density = def->density;
        f->index = (int)fixturesByIndex.size();
        fixturesByIndex.push_back(f);
        if (body->flags & kBodyActive) {                                // b2fixture.d:450-465
            f->proxyCount = 1;
            FixtureProxy* proxy = &f->proxy;
            ShapeComputeAABB(f->shape, &proxy->aabb, body->xf);
            proxy->proxyId = contactManager.broadPhase.CreateProxy(proxy->aabb, proxy);
            proxy->fixture = f;
            proxy->childIndex = 0;
        }
        f->next = body->fixtureList;
        body->fixtureList = f;
        ++body->fixtureCount;
        f->body = body;
        if (f->density > 0.0f) body->ResetMassData();
        flags |= kNewFixture;
        return f;
    }

    Joint* CreateDistance(const dbox_distance_def* def) {               // b2world.d:196-261, b2distancejoint.d:122-133
        Joint* j = new Joint();
        j->type = kDistanceJoint;
        j->bodyA = bodiesByIndex[def->body_a];
        j->bodyB = bodiesByIndex[def->body_b];
        j->collideConnected = def->collide_connected != 0;
        j->islandFlag = false;
        j->localAnchorA = Vec2(def->local_anchor_a.x, def->local_anchor_a.y);
        j->localAnchorB = Vec2(def->local_anchor_b.x, def->local_anchor_b.y);
        j->length = def->length;
        j->frequencyHz = def->frequency_hz;
        j->dampingRatio = def->damping_ratio;
        j->impulse.SetZero();
        j->gamma = 0.0f;
        j->bias = 0.0f;
        return LinkJoint(j);
    }

    Joint* CreateRope(const dbox_rope_def* def) {                       // b2ropejoint.d:140-153
        Joint* j = new Joint();
        j->type = kRopeJoint;
        j->bodyA = bodiesByIndex[def->body_a];
        j->bodyB = bodiesByIndex[def->body_b];
        j->collideConnected = def->collide_connected != 0;
        j->localAnchorA = Vec2(def->local_anchor_a.x, def->local_anchor_a.y);
        j->localAnchorB = Vec2(def->local_anchor_b.x, def->local_anchor_b.y);
        j->length = def->max_length;
        j->distMass = 0.0f;
        j->impulse.SetZero();
        j->limitState = kInactiveLimit;
        j->curLength = 0.0f;
        return LinkJoint(j);
    }

    Joint* CreateWeld(const dbox_weld_def* def) {                       // b2weldjoint.d:107-119
        Joint* j = new Joint();
        j->type = kWeldJoint;
        j->bodyA = bodiesByIndex[def->body_a];
        j->bodyB = bodiesByIndex[def->body_b];
        j->collideConnected = def->collide_connected != 0;
        j->localAnchorA = Vec2(def->local_anchor_a.x, def->local_anchor_a.y);
        j->localAnchorB = Vec2(def->local_anchor_b.x, def->local_anchor_b.y);
        j->referenceAngle = def->reference_angle;
        j->frequencyHz = def->frequency_hz;
        j->dampingRatio = def->damping_ratio;
        j->impulse.SetZero();
        return LinkJoint(j);
    }

    Joint* CreateFriction(const dbox_friction_def* def) {               // b2frictionjoint.d:85-96
        Joint* j = new Joint();
        j->type = kFrictionJoint;
        j->bodyA = bodiesByIndex[def->body_a];
        j->bodyB = bodiesByIndex[def->body_b];
        j->collideConnected = def->collide_connected != 0;
        j->localAnchorA = Vec2(def->local_anchor_a.x, def->local_anchor_a.y);
        j->localAnchorB = Vec2(def->local_anchor_b.x, def->local_anchor_b.y);
        j->impulse.SetZero();
        j->maxForce = def->max_force;
        j->maxTorque = def->max_torque;
        return LinkJoint(j);
    }

    Joint* CreateMotor(const dbox_motor_def* def) {                     // b2motorjoint.d:92-106
        Joint* j = new Joint();
        j->type = kMotorJoint;
        j->bodyA = bodiesByIndex[def->body_a];
        j->bodyB = bodiesByIndex[def->body_b];
        j->collideConnected = def->collide_connected != 0;
        j->linearOffset = Vec2(def->linear_offset.x, def->linear_offset.y);
        j->angularOffset = def->angular_offset;
        j->impulse.SetZero();
        j->maxForce = def->max_force;
        j->maxTorque = def->max_torque;
        j->correctionFactor = def->correction_factor;
        return LinkJoint(j);
    }

    Joint* CreateWheel(const dbox_wheel_def* def) {                     // b2wheeljoint.d:110-139
        Joint* j = new Joint();
        j->type = kWheelJoint;
        j->bodyA = bodiesByIndex[def->body_a];
        j->bodyB = bodiesByIndex[def->body_b];
        j->collideConnected = def->collide_connected != 0;
        j->localAnchorA = Vec2(def->local_anchor_a.x, def->local_anchor_a.y);
        j->localAnchorB = Vec2(def->local_anchor_b.x, def->local_anchor_b.y);
        j->localXAxisA = Vec2(def->local_axis_a.x, def->local_axis_a.y);
        j->localYAxisA = Cross(1.0f, j->localXAxisA);
        j->wheelMass = 0.0f;
        j->impulse.SetZero();
        j->motorMass = 0.0f;
        j->motorImpulse = 0.0f;
        j->springMass = 0.0f;
        j->maxMotorTorque = def->max_motor_torque;
        j->motorSpeed = def->motor_speed;
        j->enableMotor = def->enable_motor != 0;
        j->frequencyHz = def->frequency_hz;
        j->dampingRatio = def->damping_ratio;
        j->bias = 0.0f;
        j->gamma = 0.0f;
        j->ax.SetZero();
        j->ay.SetZero();
        return LinkJoint(j);
    }

    Joint* CreatePrismatic(const dbox_prismatic_def* def) {             // b2prismaticjoint.d:163-187
        Joint* j = new Joint();
        j->type = kPrismaticJoint;
        j->bodyA = bodiesByIndex[def->body_a];
        j->bodyB = bodiesByIndex[def->body_b];
        j->collideConnected = def->collide_connected != 0;
        j->localAnchorA = Vec2(def->local_anchor_a.x, def->local_anchor_a.y);
        j->localAnchorB = Vec2(def->local_anchor_b.x, def->local_anchor_b.y);
        j->localXAxisA = Vec2(def->local_axis_a.x, def->local_axis_a.y);
        j->localXAxisA.Normalize();
        j->localYAxisA = Cross(1.0f, j->localXAxisA);
        j->referenceAngle = def->reference_angle;
        j->impulse.SetZero();
        j->motorMass = 0.0f;
        j->motorImpulse = 0.0f;
        j->lowerTranslation = def->lower_translation;
        j->upperTranslation = def->upper_translation;
        j->maxMotorForce = def->max_motor_force;
        j->motorSpeed = def->motor_speed;
        j->enableLimit = def->enable_limit != 0;
        j->enableMotor = def->enable_motor != 0;
        j->limitState = kInactiveLimit;
        j->axis.SetZero();
        j->perp.SetZero();
        return LinkJoint(j);
    }

    Joint* CreatePulley(const dbox_pulley_def* def) {                   // b2pulleyjoint.d:116-131
        Joint* j = new Joint();
        j->type = kPulleyJoint;
        j->bodyA = bodiesByIndex[def->body_a];
        j->bodyB = bodiesByIndex[def->body_b];
        j->collideConnected = def->collide_connected != 0;
        j->groundAnchorA = Vec2(def->ground_anchor_a.x, def->ground_anchor_a.y);
        j->groundAnchorB = Vec2(def->ground_anchor_b.x, def->ground_anchor_b.y);
        j->localAnchorA = Vec2(def->local_anchor_a.x, def->local_anchor_a.y);
        j->localAnchorB = Vec2(def->local_anchor_b.x, def->local_anchor_b.y);
        j->ratio = def->ratio;
        j->lengthA = def->length_a;
        j->lengthB = def->length_b;
        j->constant = def->length_a + def->ratio * def->length_b;
        j->impulse.SetZero();
        return LinkJoint(j);
    }

    Joint* CreateMouse(const dbox_mouse_def* def) {                     // b2mousejoint.d:112-129
        Joint* j = new Joint();
        j->type = kMouseJoint;
        j->bodyA = bodiesByIndex[def->body_a];
        j->bodyB = bodiesByIndex[def->body_b];
        j->collideConnected = def->collide_connected != 0;
        j->targetA = Vec2(def->target.x, def->target.y);
        j->localAnchorB = MulT(j->bodyB->xf, j->targetA);
        j->maxForce = def->max_force;
        j->impulse.SetZero();
        j->frequencyHz = def->frequency_hz;
        j->dampingRatio = def->damping_ratio;
        j->beta = 0.0f;
        j->gamma = 0.0f;
        return LinkJoint(j);
    }

    Joint* CreateRevolute(const dbox_revolute_def* def) {               // b2world.d:196-261
        Joint* j = new Joint();
        j->bodyA = bodiesByIndex[def->body_a];
        j->bodyB = bodiesByIndex[def->body_b];
        j->collideConnected = def->collide_connected != 0;
        j->islandFlag = false;
        j->localAnchorA = Vec2(def->local_anchor_a.x, def->local_anchor_a.y);
        j->localAnchorB = Vec2(def->local_anchor_b.x, def->local_anchor_b.y);
        j->referenceAngle = def->reference_angle;
        j->impulse.SetZero();
        j->motorImpulse = 0.0f;
        j->lowerAngle = def->lower_angle;
        j->upperAngle = def->upper_angle;
        j->maxMotorTorque = def->max_motor_torque;
        j->motorSpeed = def->motor_speed;
        j->enableLimit = def->enable_limit != 0;
        j->enableMotor = def->enable_motor != 0;
        j->limitState = kInactiveLimit;
        return LinkJoint(j);
    }

    // the joint into the world's list and both bodies' edge lists, and the contact filter
    // flag when the bodies may not collide (b2world.d:206-258)
    // b2World.CreateJoint (b2world.d:196-261); flagA / flagB are the definition's bodies whose
    // contacts get flagged (the joint's own bodies unless a gear joint overrode them)
    Joint* LinkJoint(Joint* j, Body* flagA = nullptr, Body* flagB = nullptr) {
        if (!flagA) flagA = j->bodyA;
        if (!flagB) flagB = j->bodyB;
        j->prev = nullptr;
        j->next = jointList;
        if (jointList) jointList->prev = j;
        jointList = j;
        ++jointCount;
        j->edgeA.joint = j;
        j->edgeA.other = j->bodyB;
        j->edgeA.prev = nullptr;
        j->edgeA.next = j->bodyA->jointList;
        if (j->bodyA->jointList) j->bodyA->jointList->prev = &j->edgeA;
        j->bodyA->jointList = &j->edgeA;
        j->edgeB.joint = j;
        j->edgeB.other = j->bodyA;
        j->edgeB.prev = nullptr;
        j->edgeB.next = j->bodyB->jointList;
        if (j->bodyB->jointList) j->bodyB->jointList->prev = &j->edgeB;
        j->bodyB->jointList = &j->edgeB;
        if (!j->collideConnected) {
            for (ContactEdge* edge = flagB->contactList; edge; edge = edge->next) {
                if (edge->other == flagA) edge->contact->flags |= kContactFilter;
            }
        }
        j->index = (int)jointsByIndex.size();
        jointsByIndex.push_back(j);
        return j;
    }

    Joint* CreateGear(const dbox_gear_def* def) {                       // b2gearjoint.d:83-168
        Joint* j = new Joint();
        j->type = kGearJoint;
        j->joint1 = jointsByIndex[def->joint1];
        j->joint2 = jointsByIndex[def->joint2];
        j->typeA = j->joint1->type;
        j->typeB = j->joint2->type;
        j->collideConnected = def->collide_connected != 0;
        f32 coordinateA = 0, coordinateB = 0;
        j->bodyC = j->joint1->bodyA;
        j->bodyA = j->joint1->bodyB;
        Transform xfA = j->bodyA->xf, xfC = j->bodyC->xf;
        f32 aA = j->bodyA->sweep.a, aC = j->bodyC->sweep.a;
        j->localAnchorC = j->joint1->localAnchorA;
        j->localAnchorA = j->joint1->localAnchorB;
        j->referenceAngleA = j->joint1->referenceAngle;
        if (j->typeA == kRevoluteJoint) {
            j->localAxisC.SetZero();
            coordinateA = aA - aC - j->referenceAngleA;
        } else {
            j->localAxisC = j->joint1->localXAxisA;
            Vec2 pC = j->localAnchorC;
            Vec2 pA = MulT(xfC.q, Mul(xfA.q, j->localAnchorA) + (xfA.p - xfC.p));
            coordinateA = Dot(pA - pC, j->localAxisC);
        }
        j->bodyD = j->joint2->bodyA;
        j->bodyB = j->joint2->bodyB;
        Transform xfB = j->bodyB->xf, xfD = j->bodyD->xf;
        f32 aB = j->bodyB->sweep.a, aD = j->bodyD->sweep.a;
        j->localAnchorD = j->joint2->localAnchorA;
        j->localAnchorB = j->joint2->localAnchorB;
        j->referenceAngleB = j->joint2->referenceAngle;
        if (j->typeB == kRevoluteJoint) {
            j->localAxisD.SetZero();
            coordinateB = aB - aD - j->referenceAngleB;
        } else {
            j->localAxisD = j->joint2->localXAxisA;
            Vec2 pD = j->localAnchorD;
            Vec2 pB = MulT(xfD.q, Mul(xfB.q, j->localAnchorB) + (xfB.p - xfD.p));
            coordinateB = Dot(pB - pD, j->localAxisD);
        }
        j->ratio = def->ratio;
        j->constant = coordinateA + j->ratio * coordinateB;
        j->impulse.SetZero();
        return LinkJoint(j, bodiesByIndex[def->body_a], bodiesByIndex[def->body_b]);
    }

    void DestroyJoint(Joint* j) {                                        // b2world.d:265-360
        const bool collideConnected = j->collideConnected;
        if (j->prev) j->prev->next = j->next;
        if (j->next) j->next->prev = j->prev;
        if (j == jointList) jointList = j->next;
        Body* bodyA = j->bodyA;
        Body* bodyB = j->bodyB;
        bodyA->SetAwake(true);
        bodyB->SetAwake(true);
        if (j->edgeA.prev) j->edgeA.prev->next = j->edgeA.next;
        if (j->edgeA.next) j->edgeA.next->prev = j->edgeA.prev;
        if (&j->edgeA == bodyA->jointList) bodyA->jointList = j->edgeA.next;
        if (j->edgeB.prev) j->edgeB.prev->next = j->edgeB.next;
        if (j->edgeB.next) j->edgeB.next->prev = j->edgeB.prev;
        if (&j->edgeB == bodyB->jointList) bodyB->jointList = j->edgeB.next;
        jointsByIndex[j->index] = nullptr;
        delete j;
        --jointCount;
        if (!collideConnected) {
            for (ContactEdge* edge = bodyB->contactList; edge; edge = edge->next)
                if (edge->other == bodyA) edge->contact->flags |= kContactFilter;
        }
    }

    // The fixtures that are one reference fixture: a chain's child edges, else the fixture.
    TableFilter tableFilter;

    // b2Fixture.Refilter (b2fixture.d:140-180): flag the fixture's contacts for filtering and
    // touch its proxies (a chain's children, as the chain fixture's proxies)
    void Refilter(Fixture* f) {
        for (ContactEdge* e = f->body->contactList; e; e = e->next) {
            Contact* c = e->contact;
            if (c->fixtureA == f || c->fixtureB == f) c->flags |= kContactFilter;
        }
        for (Fixture* g : FixtureGroup(f)) {
            if (g != f)
                for (ContactEdge* e = g->body->contactList; e; e = e->next)
                    if (e->contact->fixtureA == g || e->contact->fixtureB == g) e->contact->flags |= kContactFilter;
            if (g->proxy.proxyId >= 0) contactManager.broadPhase.BufferMove(g->proxy.proxyId);
        }
    }

    std::vector<Fixture*> FixtureGroup(Fixture* f) {
        std::vector<Fixture*> g;
        if (f->chain < 0) {
            g.push_back(f);
            return g;
        }
        const ChainRec& c = chains[f->chain];
        for (int i = 0; i + 1 < (int)c.vertices.size(); ++i) g.push_back(fixturesByIndex[c.first + i]);
        return g;
    }

    // b2Fixture.DestroyProxies (b2fixture.d:467-478) for a group, in child order, then free it.
    void FreeFixtureGroup(const std::vector<Fixture*>& g, bool proxies) {
        for (Fixture* f : g) {
            if (proxies && f->proxyCount > 0) {
                contactManager.broadPhase.DestroyProxy(f->proxy.proxyId);
                f->proxy.proxyId = -1;
                f->proxyCount = 0;
            }
        }
        for (Fixture* f : g) {
            fixturesByIndex[f->index] = nullptr;
            delete f;
        }
    }

    void DestroyFixture(Fixture* fixture) {                              // b2body.d:179-247
        Body* b = fixture->body;
        std::vector<Fixture*> g = FixtureGroup(fixture);
        auto inGroup = [&](const Fixture* f) { return std::find(g.begin(), g.end(), f) != g.end(); };
        Fixture** node = &b->fixtureList;                               // unlink from the body's list
        while (*node) {
            if (inGroup(*node)) *node = (*node)->next;
            else node = &(*node)->next;
        }
        ContactEdge* edge = b->contactList;
        while (edge) {
            Contact* c = edge->contact;
            edge = edge->next;
            if (inGroup(c->fixtureA) || inGroup(c->fixtureB)) contactManager.Destroy(c);
        }
        FreeFixtureGroup(g, (b->flags & kBodyActive) != 0);
        --b->fixtureCount;
        b->ResetMassData();
    }

    void DestroyBody(Body* b) {                                         // b2world.d:105-193
        JointEdge* je = b->jointList;
        while (je) {
            JointEdge* je0 = je;
            je = je->next;
            DestroyJoint(je0->joint);
            b->jointList = je;
        }
        b->jointList = nullptr;
        ContactEdge* ce = b->contactList;
        while (ce) {
            ContactEdge* ce0 = ce;
            ce = ce->next;
            contactManager.Destroy(ce0->contact);
        }
        b->contactList = nullptr;
        Fixture* f = b->fixtureList;
        while (f) {
            std::vector<Fixture*> g = FixtureGroup(f);
            while (f && std::find(g.begin(), g.end(), f) != g.end()) f = f->next;   // a chain is one fixture
            FreeFixtureGroup(g, true);
            b->fixtureList = f;
            --b->fixtureCount;
        }
        b->fixtureList = nullptr;
        b->fixtureCount = 0;
        if (b->prev) b->prev->next = b->next;
        if (b->next) b->next->prev = b->prev;
        if (b == bodyList) bodyList = b->next;
        --bodyCount;
        bodiesByIndex[b->index] = nullptr;
        delete b;
    }

    void Step(f32 dt, int velocityIterations, int positionIterations) { // b2world.d:367-434
        recorder.record = recording;
        contactManager.listener = (recording || recorder.presolve) ? &recorder : nullptr;
        lastToiEvents = 0;
        lastIslands = 0;
        if (flags & kNewFixture) {
            contactManager.FindNewContacts();
            flags &= ~kNewFixture;
        }
        flags |= kLocked;
        TimeStep step;
        step.dt = dt;
        step.velocityIterations = velocityIterations;
        step.positionIterations = positionIterations;
        if (dt > 0.0f) step.inv_dt = 1.0f / dt; else step.inv_dt = 0.0f;
        step.dtRatio = inv_dt0 * dt;
        step.warmStarting = warmStarting;
        contactManager.Collide();
        if (stepComplete && step.dt > 0.0f) Solve(step);
        if (continuousPhysics && step.dt > 0.0f) {
            recorder.inToi = true;
            SolveTOI(step);
            recorder.inToi = false;
        }
        if (step.dt > 0.0f) inv_dt0 = step.inv_dt;
        if (flags & kClearForces) {
            for (Body* b = bodyList; b; b = b->next) { b->force.SetZero(); b->torque = 0.0f; }
        }
        flags &= ~kLocked;
    }

    void Solve(const TimeStep& step) {                                  // b2world.d:930-1124
        Island island;
        island.listener = contactManager.listener;
        for (Body* b = bodyList; b; b = b->next) b->flags &= ~kBodyIsland;
        for (Contact* c = contactManager.contactList; c; c = c->next) c->flags &= ~kContactIsland;
        for (Joint* j = jointList; j; j = j->next) j->islandFlag = false;
        std::vector<Body*> stack;
        stack.reserve(bodyCount);
        for (Body* seed = bodyList; seed; seed = seed->next) {
            if (seed->flags & kBodyIsland) continue;
            if (seed->IsAwake() == false || seed->IsActive() == false) continue;
            if (seed->type == kStaticBody) continue;
            island.Clear();
            stack.clear();
            stack.push_back(seed);
            seed->flags |= kBodyIsland;
            while (!stack.empty()) {
                Body* b = stack.back();
                stack.pop_back();
                island.Add(b);
                b->SetAwake(true);
                if (b->type == kStaticBody) continue;
                for (ContactEdge* ce = b->contactList; ce; ce = ce->next) {
                    Contact* contact = ce->contact;
                    if (contact->flags & kContactIsland) continue;
                    if (contact->IsEnabled() == false || contact->IsTouching() == false) continue;
                    bool sensorA = contact->fixtureA->isSensor;
                    bool sensorB = contact->fixtureB->isSensor;
                    if (sensorA || sensorB) continue;
                    island.Add(contact);
                    contact->flags |= kContactIsland;
                    Body* other = ce->other;
                    if (other->flags & kBodyIsland) continue;
                    stack.push_back(other);
                    other->flags |= kBodyIsland;
                }
                for (JointEdge* je = b->jointList; je; je = je->next) {
                    if (je->joint->islandFlag == true) continue;
                    Body* other = je->other;
                    if (other->IsActive() == false) continue;
                    island.Add(je->joint);
                    je->joint->islandFlag = true;
                    if (other->flags & kBodyIsland) continue;
                    stack.push_back(other);
                    other->flags |= kBodyIsland;
                }
            }
            island.Solve(step, gravity, allowSleep);
            ++lastIslands;
            for (Body* b : island.bodies) {
                if (b->type == kStaticBody) b->flags &= ~kBodyIsland;
            }
        }
        for (Body* b = bodyList; b; b = b->next) {
            if ((b->flags & kBodyIsland) == 0) continue;
            if (b->type == kStaticBody) continue;
            b->SynchronizeFixtures();
        }
        contactManager.FindNewContacts();
    }

    void SolveTOI(const TimeStep& step) {                               // b2world.d:1127-1452
        Island island;
        island.listener = contactManager.listener;
        if (stepComplete) {
            for (Body* b = bodyList; b; b = b->next) { b->flags &= ~kBodyIsland; b->sweep.alpha0 = 0.0f; }
            for (Contact* c = contactManager.contactList; c; c = c->next) {
                c->flags &= ~(kContactToi | kContactIsland);
                c->toiCount = 0;
                c->toi = 1.0f;
            }
        }
        for (;;) {
            Contact* minContact = nullptr;
            f32 minAlpha = 1.0f;
            for (Contact* c = contactManager.contactList; c; c = c->next) {
                if (c->IsEnabled() == false) continue;
                if (c->toiCount > kMaxSubSteps) continue;
                f32 alpha = 1.0f;
                if (c->flags & kContactToi) {
                    alpha = c->toi;
                } else {
                    Fixture* fA = c->fixtureA;
                    Fixture* fB = c->fixtureB;
                    if (fA->isSensor || fB->isSensor) continue;
                    Body* bA = fA->body;
                    Body* bB = fB->body;
                    int typeA = bA->type;
                    int typeB = bB->type;
                    bool activeA = bA->IsAwake() && typeA != kStaticBody;
                    bool activeB = bB->IsAwake() && typeB != kStaticBody;
                    if (activeA == false && activeB == false) continue;
                    bool collideA = bA->IsBullet() || typeA != kDynamicBody;
                    bool collideB = bB->IsBullet() || typeB != kDynamicBody;
                    if (collideA == false && collideB == false) continue;
                    f32 alpha0 = bA->sweep.alpha0;
                    if (bA->sweep.alpha0 < bB->sweep.alpha0) {
                        alpha0 = bB->sweep.alpha0;
                        bA->sweep.Advance(alpha0);
                    } else if (bB->sweep.alpha0 < bA->sweep.alpha0) {
                        alpha0 = bA->sweep.alpha0;
                        bB->sweep.Advance(alpha0);
                    }
                    TOIInput input;
                    input.proxyA.Set(fA->shape);
                    input.proxyB.Set(fB->shape);
                    input.sweepA = bA->sweep;
                    input.sweepB = bB->sweep;
                    input.tMax = 1.0f;
                    TOIOutput output;
                    TimeOfImpact(&output, &input);
                    f32 beta = output.t;
                    if (output.state == kToiTouching) alpha = Min(alpha0 + (1.0f - alpha0) * beta, 1.0f);
                    else alpha = 1.0f;
                    c->toi = alpha;
                    c->flags |= kContactToi;
                }
                if (alpha < minAlpha) { minContact = c; minAlpha = alpha; }
            }
            if (minContact == nullptr || 1.0f - 10.0f * kEpsilon < minAlpha) {
                stepComplete = true;
                break;
            }
            ++lastToiEvents;
            Fixture* fA = minContact->fixtureA;
            Fixture* fB = minContact->fixtureB;
            Body* bA = fA->body;
            Body* bB = fB->body;
            Sweep backup1 = bA->sweep;
            Sweep backup2 = bB->sweep;
            bA->Advance(minAlpha);
            bB->Advance(minAlpha);
            minContact->Update(contactManager.listener);
            minContact->flags &= ~kContactToi;
            ++minContact->toiCount;
            if (minContact->IsEnabled() == false || minContact->IsTouching() == false) {
                minContact->SetEnabled(false);
                bA->sweep = backup1;
                bB->sweep = backup2;
                bA->SynchronizeTransform();
                bB->SynchronizeTransform();
                continue;
            }
            bA->SetAwake(true);
            bB->SetAwake(true);
            island.Clear();
            island.Add(bA);
            island.Add(bB);
            island.Add(minContact);
            bA->flags |= kBodyIsland;
            bB->flags |= kBodyIsland;
            minContact->flags |= kContactIsland;
            Body* bodies2[2] = {bA, bB};
            for (int i = 0; i < 2; ++i) {
                Body* body = bodies2[i];
                if (body->type == kDynamicBody) {
                    for (ContactEdge* ce = body->contactList; ce; ce = ce->next) {
                        if ((int)island.bodies.size() == 2 * kMaxTOIContacts) break;
                        if ((int)island.contacts.size() == kMaxTOIContacts) break;
                        Contact* contact = ce->contact;
                        if (contact->flags & kContactIsland) continue;
                        Body* other = ce->other;
                        if (other->type == kDynamicBody && body->IsBullet() == false && other->IsBullet() == false) continue;
                        bool sensorA = contact->fixtureA->isSensor;
                        bool sensorB = contact->fixtureB->isSensor;
                        if (sensorA || sensorB) continue;
                        Sweep backup = other->sweep;
                        if ((other->flags & kBodyIsland) == 0) other->Advance(minAlpha);
                        contact->Update(contactManager.listener);
                        if (contact->IsEnabled() == false) {
                            other->sweep = backup;
                            other->SynchronizeTransform();
                            continue;
                        }
                        if (contact->IsTouching() == false) {
                            other->sweep = backup;
                            other->SynchronizeTransform();
                            continue;
                        }
                        contact->flags |= kContactIsland;
                        island.Add(contact);
                        if (other->flags & kBodyIsland) continue;
                        other->flags |= kBodyIsland;
                        if (other->type != kStaticBody) other->SetAwake(true);
                        island.Add(other);
                    }
                }
            }
            TimeStep subStep;
            subStep.dt = (1.0f - minAlpha) * step.dt;
            subStep.inv_dt = 1.0f / subStep.dt;
            subStep.dtRatio = 1.0f;
            subStep.positionIterations = 20;
            subStep.velocityIterations = step.velocityIterations;
            subStep.warmStarting = false;
            island.SolveTOI(subStep, bA->islandIndex, bB->islandIndex);
            for (Body* body : island.bodies) {
                body->flags &= ~kBodyIsland;
                if (body->type != kDynamicBody) continue;
                body->SynchronizeFixtures();
                for (ContactEdge* ce = body->contactList; ce; ce = ce->next) {
                    ce->contact->flags &= ~(kContactToi | kContactIsland);
                }
            }
            contactManager.FindNewContacts();
            if (subStepping) { stepComplete = false; break; }
        }
    }
};

void Body::SynchronizeFixtures() {                                      // b2body.d:1129-1141, b2fixture.d:480-502
    Transform xf1;
    xf1.q.Set(sweep.a0);
    xf1.p = sweep.c0 - Mul(xf1.q, sweep.localCenter);
    BroadPhase* broadPhase = &world->contactManager.broadPhase;
    for (Fixture* f = fixtureList; f; f = f->next) {
        if (f->proxyCount == 0) continue;
        FixtureProxy* proxy = &f->proxy;
        AABB aabb1, aabb2;
        ShapeComputeAABB(f->shape, &aabb1, xf1);
        ShapeComputeAABB(f->shape, &aabb2, xf);
        proxy->aabb.Combine(aabb1, aabb2);
        Vec2 displacement = xf.p - xf1.p;
        broadPhase->MoveProxy(proxy->proxyId, proxy->aabb, displacement);
    }
}

void Body::ResetMassData() {                                            // b2body.d:555-625
    mass = 0.0f;
    invMass = 0.0f;
    I = 0.0f;
    invI = 0.0f;
    sweep.localCenter.SetZero();
    if (type == kStaticBody || type == kKinematicBody) {
        sweep.c0 = xf.p;
        sweep.c = xf.p;
        sweep.a0 = sweep.a;
        return;
    }
    Vec2 localCenter(0.0f, 0.0f);
    for (Fixture* f = fixtureList; f; f = f->next) {
        if (f->density == 0.0f) continue;
        MassData massData;
        ShapeComputeMass(f->shape, &massData, f->density);
        mass += massData.mass;
        localCenter += massData.mass * massData.center;
        I += massData.I;
    }
    if (mass > 0.0f) {
        invMass = 1.0f / mass;
        localCenter *= invMass;
    } else {
        mass = 1.0f;
        invMass = 1.0f;
    }
    if (I > 0.0f && (flags & kBodyFixedRotation) == 0) {
        I -= mass * Dot(localCenter, localCenter);
        invI = 1.0f / I;
    } else {
        I = 0.0f;
        invI = 0.0f;
    }
    Vec2 oldCenter = sweep.c;
    sweep.localCenter = localCenter;
    sweep.c0 = sweep.c = Mul(xf, sweep.localCenter);
    linearVelocity += Cross(angularVelocity, sweep.c - oldCenter);
}

static bool BuildShape(const dbox_shape_def* sd, Shape* s) {
    switch (sd->kind) {
    case DBOX_SHAPE_CIRCLE:
        s->type = kCircle;
        s->radius = sd->radius;
        s->p = Vec2(sd->center.x, sd->center.y);
        return true;
    case DBOX_SHAPE_POLYGON: {
        s->type = kPolygon;
        s->radius = kPolygonRadius;
        s->count = 0;
        s->centroid.SetZero();
        Vec2 vs[kMaxPolygonVertices];
        int n = sd->count < kMaxPolygonVertices ? sd->count : kMaxPolygonVertices;
        for (int i = 0; i < n; ++i) vs[i] = Vec2(sd->vertices[i].x, sd->vertices[i].y);
        return PolygonSet(s, vs, n);
    }
    case DBOX_SHAPE_BOX:
        s->type = kPolygon;
        s->radius = kPolygonRadius;
        PolygonSetAsBox(s, sd->hx, sd->hy);
        return true;
    case DBOX_SHAPE_ORIENTED_BOX:
        s->type = kPolygon;
        s->radius = kPolygonRadius;
        PolygonSetAsBox(s, sd->hx, sd->hy, Vec2(sd->center.x, sd->center.y), sd->angle);
        return true;
    case DBOX_SHAPE_EDGE:                                               // b2EdgeShape.Set + ghost vertices
        s->type = kEdge;
        s->radius = kPolygonRadius;
        s->count = 2;
        s->vertices[0] = Vec2(sd->vertices[0].x, sd->vertices[0].y);
        s->vertices[1] = Vec2(sd->vertices[1].x, sd->vertices[1].y);
        s->hasVertex0 = (sd->count & 1) != 0;
        s->hasVertex3 = (sd->count & 2) != 0;
        s->vertex0 = s->hasVertex0 ? Vec2(sd->vertices[2].x, sd->vertices[2].y) : Vec2(0.0f, 0.0f);
        s->vertex3 = s->hasVertex3 ? Vec2(sd->vertices[3].x, sd->vertices[3].y) : Vec2(0.0f, 0.0f);
        return true;
    default:
        return false;
    }
}

}  // namespace orc

using namespace orc;

struct orc_world { World w; };

// ------------------------------------------------------------ b2World.Dump
// The text b2World.Dump logs (b2world.d:796-855, b2body.d:992-1022, b2fixture.d:280-358 and the
// joints' Dump): D statements that rebuild the world, every float as %.15e with an 'f' suffix.
struct DumpText {
    std::string s;
    void put(const char* fmt, ...) __attribute__((format(printf, 2, 3))) {
        char tmp[512];
        va_list ap;
        va_start(ap, fmt);
        int n = vsnprintf(tmp, sizeof(tmp), fmt, ap);
        va_end(ap);
        s.append(tmp, n < (int)sizeof(tmp) ? n : (int)sizeof(tmp) - 1);
    }
    void vec(const char* indent, const char* what, Vec2 v) { put("%s%s.Set(%.15ef, %.15ef);\n", indent, what, (double)v.x, (double)v.y); }
    void num(const char* indent, const char* what, f32 v) { put("%s%s = %.15ef;\n", indent, what, (double)v); }
    void flag(const char* indent, const char* what, int v) { put("%s%s = bool(%d);\n", indent, what, v); }
};

static void DumpFixture(DumpText& t, const World& w, const Fixture* f, int bodyIndex) {   // b2fixture.d:280-358
    const char* in = "    ";
    const bool chain = f->chain >= 0;
    t.put("    b2FixtureDef fd;\n");
    t.num(in, "fd.friction", f->friction);
    t.num(in, "fd.restitution", f->restitution);
    t.num(in, "fd.density", chain ? w.chains[f->chain].density : f->density);
    t.put("    fd.isSensor = bool(%d);\n", f->isSensor ? 1 : 0);
    t.put("    fd.filter.categoryBits = uint16(%d);\n", (int)f->filter.categoryBits);
    t.put("    fd.filter.maskBits = uint16(%d);\n", (int)f->filter.maskBits);
    t.put("    fd.filter.groupIndex = int16(%d);\n", (int)f->filter.groupIndex);
    const Shape& s = f->shape;
    if (chain) {
        const ChainRec& c = w.chains[f->chain];
        const int n = (int)c.vertices.size();
        t.put("    b2ChainShape shape;\n");
        t.put("    b2Vec2 vs[%d];\n", n);
        for (int i = 0; i < n; ++i)
            t.put("    vs[%d].Set(%.15ef, %.15ef);\n", i, (double)c.vertices[i].x, (double)c.vertices[i].y);
        t.put("    shape.CreateChain(vs, %d);\n", n);
        t.vec(in, "shape.m_prevVertex", c.prevVertex);
        t.vec(in, "shape.m_nextVertex", c.nextVertex);
        t.flag(in, "shape.m_hasPrevVertex", c.hasPrevVertex ? 1 : 0);
        t.flag(in, "shape.m_hasNextVertex", c.hasNextVertex ? 1 : 0);
    } else if (s.type == kCircle) {
        t.put("    b2CircleShape shape;\n");
        t.num(in, "shape.m_radius", s.radius);
        t.vec(in, "shape.m_p", s.p);
    } else if (s.type == kEdge) {
        t.put("    b2EdgeShape shape;\n");
        t.num(in, "shape.m_radius", s.radius);
        t.vec(in, "shape.m_vertex0", s.vertex0);
        t.vec(in, "shape.m_vertex1", s.vertices[0]);
        t.vec(in, "shape.m_vertex2", s.vertices[1]);
        t.vec(in, "shape.m_vertex3", s.vertex3);
        t.flag(in, "shape.m_hasVertex0", s.hasVertex0 ? 1 : 0);
        t.flag(in, "shape.m_hasVertex3", s.hasVertex3 ? 1 : 0);
    } else {
        t.put("    b2PolygonShape shape;\n");
        t.put("    b2Vec2 vs[%d];\n", kMaxPolygonVertices);
        for (int i = 0; i < s.count; ++i)
            t.put("    vs[%d].Set(%.15ef, %.15ef);\n", i, (double)s.vertices[i].x, (double)s.vertices[i].y);
        t.put("    shape.Set(vs, %d);\n", s.count);
    }
    t.put("\n");
    t.put("    fd.shape = &shape;\n");
    t.put("\n");
    t.put("    bodies[%d].CreateFixture(&fd);\n", bodyIndex);
}

static void DumpJoint(DumpText& t, const Joint* j) {                    // the joints' Dump
    static const char* names[] = {"b2RevoluteJointDef", "b2DistanceJointDef", "b2RopeJointDef", "b2WeldJointDef",
                                  "b2FrictionJointDef", "b2MotorJointDef", "b2WheelJointDef", "b2PrismaticJointDef",
                                  "b2PulleyJointDef", "", "b2GearJointDef"};
    if (j->type == kMouseJoint) {                                       // b2mousejoint.d:180-183
        t.put("Mouse joint dumping is not supported.\n");
        return;
    }
    const char* in = "  ";
    t.put("  %s jd;\n", names[j->type]);
    t.put("  jd.bodyA = bodies[%d];\n", j->bodyA->islandIndex);
    t.put("  jd.bodyB = bodies[%d];\n", j->bodyB->islandIndex);
    t.flag(in, "jd.collideConnected", j->collideConnected ? 1 : 0);
    switch (j->type) {
    case kGearJoint:                                                    // b2gearjoint.d:222-238
        t.put("  jd.joint1 = joints[%d];\n", j->joint1->dumpIndex);
        t.put("  jd.joint2 = joints[%d];\n", j->joint2->dumpIndex);
        t.num(in, "jd.ratio", j->ratio);
        break;
    case kRevoluteJoint:                                                // b2revolutejoint.d:293-312
        t.vec(in, "jd.localAnchorA", j->localAnchorA);
        t.vec(in, "jd.localAnchorB", j->localAnchorB);
        t.num(in, "jd.referenceAngle", j->referenceAngle);
        t.flag(in, "jd.enableLimit", j->enableLimit ? 1 : 0);
        t.num(in, "jd.lowerAngle", j->lowerAngle);
        t.num(in, "jd.upperAngle", j->upperAngle);
        t.flag(in, "jd.enableMotor", j->enableMotor ? 1 : 0);
        t.num(in, "jd.motorSpeed", j->motorSpeed);
        t.num(in, "jd.maxMotorTorque", j->maxMotorTorque);
        break;
    case kDistanceJoint:                                                // b2distancejoint.d:189-203
        t.vec(in, "jd.localAnchorA", j->localAnchorA);
        t.vec(in, "jd.localAnchorB", j->localAnchorB);
        t.num(in, "jd.length", j->length);
        t.num(in, "jd.frequencyHz", j->frequencyHz);
        t.num(in, "jd.dampingRatio", j->dampingRatio);
        break;
    case kRopeJoint:                                                    // b2ropejoint.d:145-157
        t.vec(in, "jd.localAnchorA", j->localAnchorA);
        t.vec(in, "jd.localAnchorB", j->localAnchorB);
        t.num(in, "jd.maxLength", j->length);
        break;
    case kWeldJoint:                                                    // b2weldjoint.d:174-188
        t.vec(in, "jd.localAnchorA", j->localAnchorA);
        t.vec(in, "jd.localAnchorB", j->localAnchorB);
        t.num(in, "jd.referenceAngle", j->referenceAngle);
        t.num(in, "jd.frequencyHz", j->frequencyHz);
        t.num(in, "jd.dampingRatio", j->dampingRatio);
        break;
    case kFrictionJoint:                                                // b2frictionjoint.d:157-170
        t.vec(in, "jd.localAnchorA", j->localAnchorA);
        t.vec(in, "jd.localAnchorB", j->localAnchorB);
        t.num(in, "jd.maxForce", j->maxForce);
        t.num(in, "jd.maxTorque", j->maxTorque);
        break;
    case kMotorJoint:                                                   // b2motorjoint.d:201-215
        t.vec(in, "jd.linearOffset", j->linearOffset);
        t.num(in, "jd.angularOffset", j->angularOffset);
        t.num(in, "jd.maxForce", j->maxForce);
        t.num(in, "jd.maxTorque", j->maxTorque);
        t.num(in, "jd.correctionFactor", j->correctionFactor);
        break;
    case kWheelJoint:                                                   // b2wheeljoint.d:277-294
        t.vec(in, "jd.localAnchorA", j->localAnchorA);
        t.vec(in, "jd.localAnchorB", j->localAnchorB);
        t.vec(in, "jd.localAxisA", j->localXAxisA);
        t.flag(in, "jd.enableMotor", j->enableMotor ? 1 : 0);
        t.num(in, "jd.motorSpeed", j->motorSpeed);
        t.num(in, "jd.maxMotorTorque", j->maxMotorTorque);
        t.num(in, "jd.frequencyHz", j->frequencyHz);
        t.num(in, "jd.dampingRatio", j->dampingRatio);
        break;
    case kPrismaticJoint:                                               // b2prismaticjoint.d:364-383
        t.vec(in, "jd.localAnchorA", j->localAnchorA);
        t.vec(in, "jd.localAnchorB", j->localAnchorB);
        t.vec(in, "jd.localAxisA", j->localXAxisA);
        t.num(in, "jd.referenceAngle", j->referenceAngle);
        t.flag(in, "jd.enableLimit", j->enableLimit ? 1 : 0);
        t.num(in, "jd.lowerTranslation", j->lowerTranslation);
        t.num(in, "jd.upperTranslation", j->upperTranslation);
        t.flag(in, "jd.enableMotor", j->enableMotor ? 1 : 0);
        t.num(in, "jd.motorSpeed", j->motorSpeed);
        t.num(in, "jd.maxMotorForce", j->maxMotorForce);
        break;
    case kPulleyJoint:                                                  // b2pulleyjoint.d:207-223
        t.vec(in, "jd.groundAnchorA", j->groundAnchorA);
        t.vec(in, "jd.groundAnchorB", j->groundAnchorB);
        t.vec(in, "jd.localAnchorA", j->localAnchorA);
        t.vec(in, "jd.localAnchorB", j->localAnchorB);
        t.num(in, "jd.lengthA", j->lengthA);
        t.num(in, "jd.lengthB", j->lengthB);
        t.num(in, "jd.ratio", j->ratio);
        break;
    }
    t.put("  joints[%d] = m_world.CreateJoint(&jd);\n", j->dumpIndex);
}

static std::string DumpWorld(World& w) {                                // b2world.d:796-855
    DumpText t;
    if (w.flags & World::kLocked) return t.s;
    t.put("b2Vec2 g(%.15ef, %.15ef);\n", (double)w.gravity.x, (double)w.gravity.y);
    t.put("m_world.SetGravity(g);\n");
    t.put("b2Body** bodies = cast(b2Body**)b2Alloc(%d * (b2Body*).sizeof);\n", w.bodyCount);
    t.put("b2Joint joints = cast(b2Joint)b2Alloc(%d * (b2Joint).sizeof);\n", w.jointCount);
    int i = 0;
    for (Body* b = w.bodyList; b; b = b->next, ++i) {                   // b2body.d:992-1022
        b->islandIndex = i;
        const char* in = "  ";
        t.put("{\n");
        t.put("  b2BodyDef bd;\n");
        t.put("  bd.type = b2BodyType(%d);\n", b->type);
        t.vec(in, "bd.position", b->xf.p);
        t.num(in, "bd.angle", b->sweep.a);
        t.vec(in, "bd.linearVelocity", b->linearVelocity);
        t.num(in, "bd.angularVelocity", b->angularVelocity);
        t.num(in, "bd.linearDamping", b->linearDamping);
        t.num(in, "bd.angularDamping", b->angularDamping);
        t.flag(in, "bd.allowSleep", b->flags & kBodyAutoSleep);
        t.flag(in, "bd.awake", b->flags & kBodyAwake);
        t.flag(in, "bd.fixedRotation", b->flags & kBodyFixedRotation);
        t.flag(in, "bd.bullet", b->flags & kBodyBullet);
        t.flag(in, "bd.active", b->flags & kBodyActive);
        t.num(in, "bd.gravityScale", b->gravityScale);
        t.put("  bodies[%d] = m_world.CreateBody(&bd);\n", i);
        t.put("\n");
        int lastChain = -1;
        for (Fixture* f = b->fixtureList; f; f = f->next) {
            if (f->chain >= 0 && f->chain == lastChain) continue;       // one fixture per chain
            lastChain = f->chain;
            t.put("  {\n");
            DumpFixture(t, w, f, i);
            t.put("  }\n");
        }
        t.put("}\n");
    }
    i = 0;
    for (Joint* j = w.jointList; j; j = j->next) j->dumpIndex = i++;    // b2Joint.m_index
    for (int pass = 0; pass < 2; ++pass)                                // gear joints last
        for (Joint* j = w.jointList; j; j = j->next) {
            if ((j->type == kGearJoint) != (pass == 1)) continue;
            t.put("{\n");
            DumpJoint(t, j);
            t.put("}\n");
        }
    t.put("b2Free(joints);\n");
    t.put("b2Free(bodies);\n");
    t.put("joints = null;\n");
    t.put("bodies = null;\n");
    return t.s;
}

// ------------------------------------------------------------ world queries
// Shape ray casts (b2RayCastInput p1, p2, maxFraction -> fraction, normal).
static bool RayCastCircle(const Shape& s, const Transform& xf, Vec2 p1, Vec2 p2, f32 maxFraction, f32* fraction,
                          Vec2* normal) {                               // b2circleshape.d:72-104
    Vec2 position = xf.p + Mul(xf.q, s.p);
    Vec2 d = p1 - position;
    f32 b = Dot(d, d) - s.radius * s.radius;
    Vec2 r = p2 - p1;
    f32 c = Dot(d, r);
    f32 rr = Dot(r, r);
    f32 sigma = c * c - rr * b;
    if (sigma < 0.0f || rr < kEpsilon) return false;
    f32 a = -(c + sqrtf(sigma));
    if (0.0f <= a && a <= maxFraction * rr) {
        a /= rr;
        *fraction = a;
        *normal = d + a * r;
        normal->Normalize();
        return true;
    }
    return false;
}

static bool RayCastPolygon(const Shape& s, const Transform& xf, Vec2 rp1, Vec2 rp2, f32 maxFraction, f32* fraction,
                           Vec2* normal) {                              // b2polygonshape.d:283-351
    Vec2 p1 = MulT(xf.q, rp1 - xf.p);
    Vec2 p2 = MulT(xf.q, rp2 - xf.p);
    Vec2 d = p2 - p1;
    f32 lower = 0.0f, upper = maxFraction;
    int index = -1;
    for (int i = 0; i < s.count; ++i) {
        f32 numerator = Dot(s.normals[i], s.vertices[i] - p1);
        f32 denominator = Dot(s.normals[i], d);
        if (denominator == 0.0f) {
            if (numerator < 0.0f) return false;
        } else if (denominator < 0.0f && numerator < lower * denominator) {
            lower = numerator / denominator;                            // the segment enters this half-space
            index = i;
        } else if (denominator > 0.0f && numerator < upper * denominator) {
            upper = numerator / denominator;                            // the segment leaves it
        }
        if (upper < lower) return false;
    }
    if (index >= 0) {
        *fraction = lower;
        *normal = Mul(xf.q, s.normals[index]);
        return true;
    }
    return false;
}

static bool RayCastEdge(const Shape& s, const Transform& xf, Vec2 rp1, Vec2 rp2, f32 maxFraction, f32* fraction,
                        Vec2* normal) {                                 // b2edgeshape.d:96-157
    Vec2 p1 = MulT(xf.q, rp1 - xf.p);
    Vec2 p2 = MulT(xf.q, rp2 - xf.p);
    Vec2 d = p2 - p1;
    Vec2 v1 = s.vertices[0], v2 = s.vertices[1];
    Vec2 e = v2 - v1;
    Vec2 n(e.y, -e.x);
    n.Normalize();
    f32 numerator = Dot(n, v1 - p1);
    f32 denominator = Dot(n, d);
    if (denominator == 0.0f) return false;
    f32 t = numerator / denominator;
    if (t < 0.0f || maxFraction < t) return false;
    Vec2 q = p1 + t * d;
    Vec2 r = v2 - v1;
    f32 rr = Dot(r, r);
    if (rr == 0.0f) return false;
    f32 sv = Dot(q - v1, r) / rr;
    if (sv < 0.0f || 1.0f < sv) return false;
    *fraction = t;
    Vec2 wn = Mul(xf.q, n);
    *normal = numerator > 0.0f ? Vec2(-wn.x, -wn.y) : wn;
    return true;
}

static bool RayCastFixture(const Fixture* f, Vec2 p1, Vec2 p2, f32 maxFraction, f32* fraction, Vec2* normal) {
    const Transform& xf = f->body->xf;                                  // b2fixture.d:217-220
    if (f->shape.type == kCircle) return RayCastCircle(f->shape, xf, p1, p2, maxFraction, fraction, normal);
    if (f->shape.type == kEdge) return RayCastEdge(f->shape, xf, p1, p2, maxFraction, fraction, normal);
    return RayCastPolygon(f->shape, xf, p1, p2, maxFraction, fraction, normal);
}

// b2World.QueryAABB (b2world.d:563-569) through b2WorldQueryWrapper (b2world.d:1592-1603) with a
// callback that keeps every fixture reported
struct QueryCollect {
    const DynamicTree* tree;
    std::vector<int> found;
    bool QueryCallback(int proxyId) {
        found.push_back(((const FixtureProxy*)tree->nodes[proxyId].userData)->fixture->index);
        return true;
    }
};

// b2World.RayCast (b2world.d:577-587) through b2WorldRayCastWrapper (b2world.d:1605-1629);
// clip = true is the closest-hit callback (returns the fraction), false keeps every hit (returns 1)
struct RayCollect {
    const DynamicTree* tree;
    bool clip;
    std::vector<dbox_ray_hit> hits;
    f32 RayCastCallback(Vec2 p1, Vec2 p2, f32 maxFraction, int proxyId) {
        const Fixture* f = ((const FixtureProxy*)tree->nodes[proxyId].userData)->fixture;
        f32 fraction;
        Vec2 normal;
        if (!RayCastFixture(f, p1, p2, maxFraction, &fraction, &normal)) return maxFraction;
        Vec2 point = (1.0f - fraction) * p1 + fraction * p2;
        dbox_ray_hit h;
        h.fixture = f->index;
        h.fraction = fraction;
        h.point.x = point.x;
        h.point.y = point.y;
        h.normal.x = normal.x;
        h.normal.y = normal.y;
        if (clip) {
            hits.assign(1, h);
            return fraction;
        }
        hits.push_back(h);
        return 1.0f;
    }
};

extern "C" {

// every fixture whose fat AABB overlaps [lower, upper], in fixture order; returns the count
int orc_query_aabb(orc_world* w, float lx, float ly, float ux, float uy, int* out, int cap) {
    QueryCollect cb;
    cb.tree = &w->w.contactManager.broadPhase.tree;
    AABB a;
    a.lowerBound = Vec2(lx, ly);
    a.upperBound = Vec2(ux, uy);
    cb.tree->Query(&cb, a);
    std::sort(cb.found.begin(), cb.found.end());
    for (int i = 0; i < (int)cb.found.size() && i < cap; ++i) out[i] = cb.found[i];
    return (int)cb.found.size();
}

// mode 0: the closest hit (the smallest fraction, the lower fixture index on a tie), from all
// hits; mode 1: every hit, in fixture order; mode 2: the reference's clipping closest-hit
// callback as it runs (the last hit it reports).  Returns the count; -1 for p1 == p2.
int orc_raycast(orc_world* w, float x1, float y1, float x2, float y2, int mode, dbox_ray_hit* out, int cap) {
    Vec2 p1(x1, y1), p2(x2, y2);
    if ((p2 - p1).LengthSquared() <= 0.0f) return -1;
    RayCollect cb;
    cb.tree = &w->w.contactManager.broadPhase.tree;
    cb.clip = mode == 2;
    cb.tree->RayCast(&cb, p1, p2, 1.0f);
    std::vector<dbox_ray_hit>& h = cb.hits;
    std::sort(h.begin(), h.end(), [](const dbox_ray_hit& a, const dbox_ray_hit& b) { return a.fixture < b.fixture; });
    if (mode == 0 && !h.empty()) {
        size_t best = 0;
        for (size_t i = 1; i < h.size(); ++i)
            if (h[i].fraction < h[best].fraction) best = i;             // in fixture order: ties keep the lower index
        h.assign(1, h[best]);
    }
    for (int i = 0; i < (int)h.size() && i < cap; ++i) out[i] = h[i];
    return (int)h.size();
}

// n rays through orc_raycast (mode 0 or 1), counts[n], hits[n * cap]
void orc_raycast_many(orc_world* w, int n, const float* p1, const float* p2, int mode, int* counts, dbox_ray_hit* hits,
                      int cap) {
    for (int i = 0; i < n; ++i)
        counts[i] = orc_raycast(w, p1[2 * i], p1[2 * i + 1], p2[2 * i], p2[2 * i + 1], mode, hits + (size_t)i * cap, cap);
}

// n boxes (lower x, y, upper x, y) through orc_query_aabb, counts[n], out[n * cap]
void orc_query_aabb_many(orc_world* w, int n, const float* boxes, int* counts, int* out, int cap) {
    for (int i = 0; i < n; ++i)
        counts[i] = orc_query_aabb(w, boxes[4 * i], boxes[4 * i + 1], boxes[4 * i + 2], boxes[4 * i + 3],
                                   out + (size_t)i * cap, cap);
}

// b2World.Dump into buf (NUL-terminated when it fits); returns the text's length
int orc_world_dump(orc_world* w, char* buf, int cap) {
    std::string s = DumpWorld(w->w);
    if (buf && cap > 0) {
        size_t n = s.size() < (size_t)cap - 1 ? s.size() : (size_t)cap - 1;
        memcpy(buf, s.data(), n);
        buf[n] = 0;
    }
    return (int)s.size();
}

void orc_set_trig_mode(int mode) { g_trig_mode = mode; }
int orc_get_trig_mode(void) { return g_trig_mode; }

void orc_sincos(float a, float* s, float* c) { SinCos(a, s, c); }

void orc_sincos_array(int n, const float* a, float* s, float* c) {
    for (int i = 0; i < n; ++i) SinCos(a[i], s + i, c + i);
}

orc_world* orc_world_create(float gx, float gy) {
    orc_world* w = new orc_world();
    w->w.gravity = Vec2(gx, gy);
    return w;
}

void orc_world_destroy(orc_world* w) { delete w; }

int orc_body_create(orc_world* w, const dbox_body_def* def) { return w->w.CreateBody(def)->index; }

int orc_fixture_create(orc_world* w, int body, const dbox_shape_def* shape, const dbox_fixture_def* def) {
    if (body < 0 || body >= (int)w->w.bodiesByIndex.size()) return -1;
    Shape s;
    if (!BuildShape(shape, &s)) return -1;
    if (!w->w.bodiesByIndex[body]) return -1;
    return w->w.CreateFixture(w->w.bodiesByIndex[body], s, def)->index;
}

// b2Body.CreateFixture with a b2ChainShape (b2chainshape.d: CreateChain / CreateLoop,
// SetPrevVertex / SetNextVertex) as its child edges (GetChildEdge), in child order
int orc_fixture_create_chain(orc_world* w, int body, const dbox_vec2* vertices, int count, int loop,
                             const dbox_vec2* prev, const dbox_vec2* next, const dbox_fixture_def* def) {
    if (body < 0 || body >= (int)w->w.bodiesByIndex.size() || !w->w.bodiesByIndex[body] || count < (loop ? 3 : 2))
        return -1;
    std::vector<Vec2> v;
    for (int i = 0; i < count; ++i) v.push_back(Vec2(vertices[i].x, vertices[i].y));
    bool hasPrev = !loop && prev, hasNext = !loop && next;
    Vec2 pv = hasPrev ? Vec2(prev->x, prev->y) : Vec2(0.0f, 0.0f);
    Vec2 nv = hasNext ? Vec2(next->x, next->y) : Vec2(0.0f, 0.0f);
    if (loop) {
        v.push_back(v[0]);
        pv = v[v.size() - 2];
        nv = v[1];
        hasPrev = hasNext = true;
    }
    dbox_fixture_def d = *def;
    d.density = 0.0f;                                                   // a chain has no mass
    int first = -1;
    const int m = (int)v.size();
    ChainRec rec;
    rec.vertices = v;
    rec.prevVertex = pv;
    rec.nextVertex = nv;
    rec.hasPrevVertex = hasPrev;
    rec.hasNextVertex = hasNext;
    rec.density = def->density;
    const int chain_id = (int)w->w.chains.size();
    for (int i = 0; i + 1 < m; ++i) {
        Shape s;
        s.type = kEdge;
        s.radius = kPolygonRadius;
        s.count = 2;
        s.vertices[0] = v[i];
        s.vertices[1] = v[i + 1];
        if (i > 0) { s.vertex0 = v[i - 1]; s.hasVertex0 = true; }
        else { s.vertex0 = pv; s.hasVertex0 = hasPrev; }
        if (i < m - 2) { s.vertex3 = v[i + 2]; s.hasVertex3 = true; }
        else { s.vertex3 = nv; s.hasVertex3 = hasNext; }
        if (!s.hasVertex0) s.vertex0.SetZero();
        if (!s.hasVertex3) s.vertex3.SetZero();
        Fixture* f = w->w.CreateFixture(w->w.bodiesByIndex[body], s, &d);
        f->chain = chain_id;
        if (first < 0) first = f->index;
    }
    rec.first = first;
    w->w.chains.push_back(rec);
    return first;
}

int orc_joint_create_revolute(orc_world* w, const dbox_revolute_def* def) {
    int n = (int)w->w.bodiesByIndex.size();
    if (def->body_a < 0 || def->body_a >= n || def->body_b < 0 || def->body_b >= n || def->body_a == def->body_b ||
        !w->w.bodiesByIndex[def->body_a] || !w->w.bodiesByIndex[def->body_b]) return -1;
    return w->w.CreateRevolute(def)->index;
}

int orc_joint_create_distance(orc_world* w, const dbox_distance_def* def) {
    int n = (int)w->w.bodiesByIndex.size();
    if (def->body_a < 0 || def->body_a >= n || def->body_b < 0 || def->body_b >= n || def->body_a == def->body_b ||
        !w->w.bodiesByIndex[def->body_a] || !w->w.bodiesByIndex[def->body_b]) return -1;
    return w->w.CreateDistance(def)->index;
}

int orc_joint_create_rope(orc_world* w, const dbox_rope_def* def) {
    int n = (int)w->w.bodiesByIndex.size();
    if (def->body_a < 0 || def->body_a >= n || def->body_b < 0 || def->body_b >= n || def->body_a == def->body_b ||
        !w->w.bodiesByIndex[def->body_a] || !w->w.bodiesByIndex[def->body_b]) return -1;
    return w->w.CreateRope(def)->index;
}

int orc_joint_create_weld(orc_world* w, const dbox_weld_def* def) {
    int n = (int)w->w.bodiesByIndex.size();
    if (def->body_a < 0 || def->body_a >= n || def->body_b < 0 || def->body_b >= n || def->body_a == def->body_b ||
        !w->w.bodiesByIndex[def->body_a] || !w->w.bodiesByIndex[def->body_b]) return -1;
    return w->w.CreateWeld(def)->index;
}

int orc_joint_create_friction(orc_world* w, const dbox_friction_def* def) {
    int n = (int)w->w.bodiesByIndex.size();
    if (def->body_a < 0 || def->body_a >= n || def->body_b < 0 || def->body_b >= n || def->body_a == def->body_b ||
        !w->w.bodiesByIndex[def->body_a] || !w->w.bodiesByIndex[def->body_b]) return -1;
    return w->w.CreateFriction(def)->index;
}

int orc_joint_create_motor(orc_world* w, const dbox_motor_def* def) {
    int n = (int)w->w.bodiesByIndex.size();
    if (def->body_a < 0 || def->body_a >= n || def->body_b < 0 || def->body_b >= n || def->body_a == def->body_b ||
        !w->w.bodiesByIndex[def->body_a] || !w->w.bodiesByIndex[def->body_b]) return -1;
    return w->w.CreateMotor(def)->index;
}

int orc_joint_create_wheel(orc_world* w, const dbox_wheel_def* def) {
    int n = (int)w->w.bodiesByIndex.size();
    if (def->body_a < 0 || def->body_a >= n || def->body_b < 0 || def->body_b >= n || def->body_a == def->body_b ||
        !w->w.bodiesByIndex[def->body_a] || !w->w.bodiesByIndex[def->body_b]) return -1;
    return w->w.CreateWheel(def)->index;
}

int orc_joint_create_prismatic(orc_world* w, const dbox_prismatic_def* def) {
    int n = (int)w->w.bodiesByIndex.size();
    if (def->body_a < 0 || def->body_a >= n || def->body_b < 0 || def->body_b >= n || def->body_a == def->body_b ||
        !w->w.bodiesByIndex[def->body_a] || !w->w.bodiesByIndex[def->body_b]) return -1;
    return w->w.CreatePrismatic(def)->index;
}

int orc_joint_create_pulley(orc_world* w, const dbox_pulley_def* def) {
    int n = (int)w->w.bodiesByIndex.size();
    if (def->body_a < 0 || def->body_a >= n || def->body_b < 0 || def->body_b >= n || def->body_a == def->body_b ||
        !w->w.bodiesByIndex[def->body_a] || !w->w.bodiesByIndex[def->body_b]) return -1;
    return w->w.CreatePulley(def)->index;
}

// a gear needs two live revolute or prismatic joints and live definition bodies
int orc_joint_create_gear(orc_world* w, const dbox_gear_def* def) {
    int n = (int)w->w.bodiesByIndex.size(), nj = (int)w->w.jointsByIndex.size();
    if (def->body_a < 0 || def->body_a >= n || def->body_b < 0 || def->body_b >= n || def->body_a == def->body_b ||
        !w->w.bodiesByIndex[def->body_a] || !w->w.bodiesByIndex[def->body_b]) return -1;
    for (int k : {def->joint1, def->joint2}) {
        if (k < 0 || k >= nj || !w->w.jointsByIndex[k]) return -1;
        int t = w->w.jointsByIndex[k]->type;
        if (t != kRevoluteJoint && t != kPrismaticJoint) return -1;
    }
    return w->w.CreateGear(def)->index;
}

int orc_joint_create_mouse(orc_world* w, const dbox_mouse_def* def) {
    int n = (int)w->w.bodiesByIndex.size();
    if (def->body_a < 0 || def->body_a >= n || def->body_b < 0 || def->body_b >= n || def->body_a == def->body_b ||
        !w->w.bodiesByIndex[def->body_a] || !w->w.bodiesByIndex[def->body_b]) return -1;
    return w->w.CreateMouse(def)->index;
}

// b2World.DestroyBody / DestroyJoint, b2Body.DestroyFixture (a chain child destroys its chain)
int orc_body_destroy(orc_world* w, int body) {
    if (body < 0 || body >= (int)w->w.bodiesByIndex.size() || !w->w.bodiesByIndex[body]) return -1;
    const Body* b = w->w.bodiesByIndex[body];
    // joints go newest first (b2world.d:115-131): a gear on this body goes before its joints;
    // a body carrying a gear's joint but neither of the gear's bodies would leave it dangling
    for (Joint* g : w->w.jointsByIndex)
        if (g && g->type == kGearJoint && g->bodyA != b && g->bodyB != b)
            for (const Joint* j : {g->joint1, g->joint2})
                if (j->bodyA == b || j->bodyB == b) return -1;
    w->w.DestroyBody(w->w.bodiesByIndex[body]);
    return 0;
}

int orc_fixture_destroy(orc_world* w, int fixture) {
    if (fixture < 0 || fixture >= (int)w->w.fixturesByIndex.size() || !w->w.fixturesByIndex[fixture]) return -1;
    w->w.DestroyFixture(w->w.fixturesByIndex[fixture]);
    return 0;
}

int orc_joint_destroy(orc_world* w, int joint) {
    if (joint < 0 || joint >= (int)w->w.jointsByIndex.size() || !w->w.jointsByIndex[joint]) return -1;
    for (Joint* g : w->w.jointsByIndex)                                 // a gear still uses it
        if (g && g->type == kGearJoint && (g->joint1 == w->w.jointsByIndex[joint] || g->joint2 == w->w.jointsByIndex[joint]))
            return -1;
    w->w.DestroyJoint(w->w.jointsByIndex[joint]);
    return 0;
}

int orc_joint_set_mouse_target(orc_world* w, int joint, float x, float y) {   // b2mousejoint.d:83-91
    if (joint < 0 || joint >= (int)w->w.jointsByIndex.size()) return -1;
    Joint* j = w->w.jointsByIndex[joint];
    if (!j || j->type != kMouseJoint) return -1;
    if (!j->bodyB->IsAwake()) j->bodyB->SetAwake(true);
    j->targetA = Vec2(x, y);
    return 0;
}

int orc_scene_create(orc_world* w, int n_bodies, const dbox_body_def* bodies, int n_fixtures,
                     const int* fixture_body, const dbox_shape_def* shapes, const dbox_fixture_def* fixtures,
                     int n_joints, const dbox_revolute_def* joints) {
    int base = (int)w->w.bodiesByIndex.size();
    for (int i = 0; i < n_bodies; ++i) orc_body_create(w, bodies + i);
    for (int i = 0; i < n_fixtures; ++i) {
        if (orc_fixture_create(w, base + fixture_body[i], shapes + i, fixtures + i) < 0) return -1;
    }
    for (int i = 0; i < n_joints; ++i) {
        dbox_revolute_def d = joints[i];
        d.body_a += base;
        d.body_b += base;
        if (orc_joint_create_revolute(w, &d) < 0) return -1;
    }
    return 0;
}

void orc_world_set_flags(orc_world* w, int warm, int continuous, int substep, int sleep, int autoclear) {
    World& W = w->w;
    W.warmStarting = warm != 0;
    W.continuousPhysics = continuous != 0;
    W.subStepping = substep != 0;
    bool flag = sleep != 0;
    if (flag != W.allowSleep) {                                         // b2world.d:627-643
        W.allowSleep = flag;
        if (!flag) for (Body* b = W.bodyList; b; b = b->next) b->SetAwake(true);
    }
    if (autoclear) W.flags |= World::kClearForces; else W.flags &= ~World::kClearForces;
}

void orc_world_step(orc_world* w, float dt, int vel_iters, int pos_iters) { w->w.Step(dt, vel_iters, pos_iters); }

void orc_world_step_n(orc_world* w, float dt, int vel_iters, int pos_iters, int steps) {
    for (int i = 0; i < steps; ++i) w->w.Step(dt, vel_iters, pos_iters);
}

int orc_fixture_set_filter(orc_world* w, int fixture, int category, int mask, int group) {   // b2fixture.d:132-137
    if (fixture < 0 || fixture >= (int)w->w.fixturesByIndex.size() || !w->w.fixturesByIndex[fixture]) return -1;
    Fixture* f = w->w.fixturesByIndex[fixture];
    for (Fixture* g : w->w.FixtureGroup(f)) {
        g->filter.categoryBits = (uint16_t)category;
        g->filter.maskBits = (uint16_t)mask;
        g->filter.groupIndex = (int16_t)group;
    }
    w->w.Refilter(f);
    return 0;
}

int orc_fixture_set_filter_class(orc_world* w, int fixture, int cls) {
    if (fixture < 0 || fixture >= (int)w->w.fixturesByIndex.size() || !w->w.fixturesByIndex[fixture]) return -1;
    Fixture* f = w->w.fixturesByIndex[fixture];
    for (Fixture* g : w->w.FixtureGroup(f)) g->fclass = cls;
    w->w.Refilter(f);
    return 0;
}

void orc_world_set_contact_filter(orc_world* w, const uint64_t* table, int with_default) {   // b2world.d:52-55
    if (!table) {
        w->w.contactManager.filter = &w->w.contactManager.defaultFilter;
        return;
    }
    memcpy(w->w.tableFilter.table, table, sizeof(w->w.tableFilter.table));
    w->w.tableFilter.withDefault = with_default != 0;
    w->w.contactManager.filter = &w->w.tableFilter;
}

void orc_world_set_presolve(orc_world* w, dbox_presolve_fn fn, void* user) {
    w->w.recorder.presolve = fn;
    w->w.recorder.presolve_user = user;
    w->w.contactManager.listener = (w->w.recording || fn) ? &w->w.recorder : nullptr;
}

void orc_world_record_events(orc_world* w, int enable) {               // the listener for steps and destruction
    w->w.recording = enable != 0;
    w->w.recorder.record = w->w.recording;
    w->w.contactManager.listener = (w->w.recording || w->w.recorder.presolve) ? &w->w.recorder : nullptr;
}
int orc_world_event_count(orc_world* w) { return (int)w->w.recorder.events.size(); }
int orc_world_get_events(orc_world* w, dbox_contact_event* out, int cap) {
    int n = (int)w->w.recorder.events.size();
    if (n > cap) n = cap;
    if (n > 0) memcpy(out, w->w.recorder.events.data(), sizeof(dbox_contact_event) * n);
    return n;
}
void orc_world_clear_events(orc_world* w) { w->w.recorder.events.clear(); }

int orc_world_last_toi_events(orc_world* w) { return w->w.lastToiEvents; }
int orc_world_last_islands(orc_world* w) { return w->w.lastIslands; }

int orc_world_export_state(orc_world* w, dbox_world_header* header, dbox_body_state* bodies,
                           dbox_proxy_state* proxies, dbox_contact_state* contacts, dbox_joint_state* joints) {
    World& W = w->w;
    std::vector<Contact*> cs;
    for (Contact* c = W.contactManager.contactList; c; c = c->next) cs.push_back(c);
    std::reverse(cs.begin(), cs.end());  // oldest first
    if (header) {
        header->body_count = (int)W.bodiesByIndex.size();
        header->fixture_count = (int)W.fixturesByIndex.size();
        header->contact_count = (int)cs.size();
        header->joint_count = (int)W.jointsByIndex.size();
        header->world_flags = W.flags;
        header->step_complete = W.stepComplete ? 1 : 0;
        header->inv_dt0 = W.inv_dt0;
        header->reserved = 0;
    }
    if (bodies) {
        for (size_t i = 0; i < W.bodiesByIndex.size(); ++i) {
            const Body* b = W.bodiesByIndex[i];
            dbox_body_state* o = bodies + i;
            if (!b) {                                                   // destroyed: an all-zero record
                memset(o, 0, sizeof(*o));
                continue;
            }
            o->flags = b->flags;
            o->type = b->type;
            o->xf[0] = b->xf.p.x; o->xf[1] = b->xf.p.y; o->xf[2] = b->xf.q.s; o->xf[3] = b->xf.q.c;
            o->sweep[0] = b->sweep.localCenter.x; o->sweep[1] = b->sweep.localCenter.y;
            o->sweep[2] = b->sweep.c0.x; o->sweep[3] = b->sweep.c0.y;
            o->sweep[4] = b->sweep.c.x; o->sweep[5] = b->sweep.c.y;
            o->sweep[6] = b->sweep.a0; o->sweep[7] = b->sweep.a; o->sweep[8] = b->sweep.alpha0;
            o->vel[0] = b->linearVelocity.x; o->vel[1] = b->linearVelocity.y; o->vel[2] = b->angularVelocity;
            o->force[0] = b->force.x; o->force[1] = b->force.y; o->force[2] = b->torque;
            o->sleep_time = b->sleepTime;
            o->mass[0] = b->mass; o->mass[1] = b->invMass; o->mass[2] = b->I; o->mass[3] = b->invI;
        }
    }
    if (proxies) {
        std::vector<char> moved(W.contactManager.broadPhase.tree.nodes.size(), 0);
        for (int id : W.contactManager.broadPhase.moveBuffer) if (id >= 0) moved[id] = 1;
        for (size_t i = 0; i < W.fixturesByIndex.size(); ++i) {
            const Fixture* f = W.fixturesByIndex[i];
            dbox_proxy_state* o = proxies + i;
            int id = f ? f->proxy.proxyId : -1;                         // destroyed: no proxy
            o->proxy_id = id;
            if (id >= 0) {
                const AABB& a = W.contactManager.broadPhase.tree.nodes[id].aabb;
                o->fat_aabb[0] = a.lowerBound.x; o->fat_aabb[1] = a.lowerBound.y;
                o->fat_aabb[2] = a.upperBound.x; o->fat_aabb[3] = a.upperBound.y;
                o->moved = moved[id];
            } else {
                memset(o->fat_aabb, 0, sizeof(o->fat_aabb));
                o->moved = 0;
            }
        }
    }
    if (contacts)
        for (size_t i = 0; i < cs.size(); ++i) FillContactState(cs[i], contacts + i);
    if (joints) {
        for (size_t i = 0; i < W.jointsByIndex.size(); ++i) {
            const Joint* j = W.jointsByIndex[i];
            if (!j) {                                                   // destroyed: an all-zero record
                memset(joints + i, 0, sizeof(joints[i]));
                continue;
            }
            joints[i].impulse[0] = j->impulse.x;
            joints[i].impulse[1] = j->impulse.y;
            joints[i].impulse[2] = j->impulse.z;
            joints[i].motor_impulse = j->motorImpulse;
            joints[i].limit_state = j->limitState;
        }
    }
    return 0;
}

int orc_polygon_set(const float* xy, int n, float* out_vertices, float* out_normals, float* out_centroid) {
    Shape s;
    s.type = kPolygon;
    s.radius = kPolygonRadius;
    Vec2 vs[kMaxPolygonVertices];
    if (n > kMaxPolygonVertices) n = kMaxPolygonVertices;
    for (int i = 0; i < n; ++i) vs[i] = Vec2(xy[2 * i], xy[2 * i + 1]);
    if (!PolygonSet(&s, vs, n)) return 0;
    for (int i = 0; i < s.count; ++i) {
        out_vertices[2 * i] = s.vertices[i].x; out_vertices[2 * i + 1] = s.vertices[i].y;
        out_normals[2 * i] = s.normals[i].x; out_normals[2 * i + 1] = s.normals[i].y;
    }
    out_centroid[0] = s.centroid.x;
    out_centroid[1] = s.centroid.y;
    return s.count;
}

int orc_collide(const dbox_shape_def* a, const float* xfa, const dbox_shape_def* b, const float* xfb,
                dbox_contact_state* out) {
    Shape sa, sb;
    if (!BuildShape(a, &sa) || !BuildShape(b, &sb)) return -1;
    Transform ta, tb;
    ta.p = Vec2(xfa[0], xfa[1]); ta.q.s = xfa[2]; ta.q.c = xfa[3];
    tb.p = Vec2(xfb[0], xfb[1]); tb.q.s = xfb[2]; tb.q.c = xfb[3];
    Manifold m;
    if (sa.type == kPolygon && sb.type == kPolygon) CollidePolygons(&m, sa, ta, sb, tb);
    else if (sa.type == kPolygon && sb.type == kCircle) CollidePolygonAndCircle(&m, sa, ta, sb, tb);
    else if (sa.type == kCircle && sb.type == kCircle) CollideCircles(&m, sa, ta, sb, tb);
    else return -1;
    memset(out, 0, sizeof(*out));
    out->point_count = m.pointCount;
    out->type = m.type;
    out->local_normal[0] = m.localNormal.x; out->local_normal[1] = m.localNormal.y;
    out->local_point[0] = m.localPoint.x; out->local_point[1] = m.localPoint.y;
    for (int k = 0; k < m.pointCount; ++k) {
        out->points[k].local_point[0] = m.points[k].localPoint.x;
        out->points[k].local_point[1] = m.points[k].localPoint.y;
        out->points[k].id = m.points[k].id.key;
    }
    return m.pointCount;
}

}  // extern "C"
