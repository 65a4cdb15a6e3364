// Host-side creation geometry of the GPU library: polygon hull and normals,
// mass properties and body mass reset.  Runs once per fixture at creation
// (the reference runs the same steps inside b2Body.CreateFixture); float32,
// no fused multiply-add (compiled with -ffp-contract=off).
#pragma once

#include <math.h>
#include <float.h>
#include "dbox_trig.h"

namespace hg {

struct V2 { float x, y; };
static inline V2 mk(float x, float y) { V2 v; v.x = x; v.y = y; return v; }
static inline V2 add(V2 a, V2 b) { return mk(a.x + b.x, a.y + b.y); }
static inline V2 sub(V2 a, V2 b) { return mk(a.x - b.x, a.y - b.y); }
static inline V2 scl(float s, V2 v) { return mk(s * v.x, s * v.y); }
static inline float dot(V2 a, V2 b) { return a.x * b.x + a.y * b.y; }
static inline float cross(V2 a, V2 b) { return a.x * b.y - a.y * b.x; }
static inline V2 cross_vs(V2 a, float s) { return mk(s * a.y, -s * a.x); }
static inline float len_sq(V2 v) { return v.x * v.x + v.y * v.y; }
static inline float normalize(V2& v) {                                 // b2math.d:160-175
    float length = sqrtf(v.x * v.x + v.y * v.y);
    if (length < FLT_EPSILON) return 0.0f;
    float inv = 1.0f / length;
    v.x *= inv;
    v.y *= inv;
    return length;
}
struct Rot { float s, c; };
static inline Rot rot(float a) { Rot r; dbox_sincosf(a, &r.s, &r.c); return r; }
static inline V2 rmul(Rot q, V2 v) { return mk(q.c * v.x - q.s * v.y, q.s * v.x + q.c * v.y); }
static inline V2 xmul(V2 p, Rot q, V2 v) {                             // b2Mul(b2Transform, b2Vec2)
    return mk((q.c * v.x - q.s * v.y) + p.x, (q.s * v.x + q.c * v.y) + p.y);
}

struct Poly { int count; V2 v[8]; V2 n[8]; V2 centroid; };

// b2PolygonShape.ComputeCentroid (b2polygonshape.d:506-554)
static V2 centroid(const V2* vs, int count) {
    V2 c = mk(0.0f, 0.0f);
    float area = 0.0f;
    V2 pRef = mk(0.0f, 0.0f);
    const float inv3 = 1.0f / 3.0f;
    for (int i = 0; i < count; ++i) {
        V2 p1 = pRef, p2 = vs[i], p3 = i + 1 < count ? vs[i + 1] : vs[0];
        V2 e1 = sub(p2, p1), e2 = sub(p3, p1);
        float D = cross(e1, e2);
        float triangleArea = 0.5f * D;
        area += triangleArea;
        c = add(c, scl(triangleArea * inv3, add(add(p1, p2), p3)));
    }
    float ia = 1.0f / area;
    c.x *= ia;
    c.y *= ia;
    return c;
}

static void set_as_box(Poly& p, float hx, float hy) {                  // b2polygonshape.d:220-232
    p.count = 4;
    p.v[0] = mk(-hx, -hy); p.v[1] = mk(hx, -hy); p.v[2] = mk(hx, hy); p.v[3] = mk(-hx, hy);
    p.n[0] = mk(0.0f, -1.0f); p.n[1] = mk(1.0f, 0.0f); p.n[2] = mk(0.0f, 1.0f); p.n[3] = mk(-1.0f, 0.0f);
    p.centroid = mk(0.0f, 0.0f);
}

static void set_as_box(Poly& p, float hx, float hy, V2 center, float angle) {  // b2polygonshape.d:238-262
    set_as_box(p, hx, hy);
    p.centroid = center;
    Rot q = rot(angle);
    for (int i = 0; i < p.count; ++i) {
        p.v[i] = xmul(center, q, p.v[i]);
        p.n[i] = rmul(q, p.n[i]);
    }
}

// b2PolygonShape.Set: weld, gift wrapping, normals, centroid (b2polygonshape.d:74-209).
static bool set_hull(Poly& p, const V2* vertices, int count) {
    if (count < 3 || count > 8) return false;
    V2 ps[8];
    int tempCount = 0;
    for (int i = 0; i < count; ++i) {
        V2 v = vertices[i];
        bool unique = true;
        for (int j = 0; j < tempCount; ++j) {
            V2 d = sub(v, ps[j]);
            if (dot(d, d) < 0.5f * 0.005f) { unique = false; break; }
        }
        if (unique) ps[tempCount++] = v;
    }
    int n = tempCount;
    if (n < 3) return false;
    int i0 = 0;
    float x0 = ps[0].x;
    for (int i = 1; i < n; ++i) {
        float x = ps[i].x;
        if (x > x0 || (x == x0 && ps[i].y < ps[i0].y)) { i0 = i; x0 = x; }
    }
    int hull[8];
    int m = 0, ih = i0;
    for (;;) {
        if (m >= 8) return false;
        hull[m] = ih;
        int ie = 0;
        for (int j = 1; j < n; ++j) {
            if (ie == ih) { ie = j; continue; }
            V2 r = sub(ps[ie], ps[hull[m]]);
            V2 v = sub(ps[j], ps[hull[m]]);
            float c = cross(r, v);
            if (c < 0.0f) ie = j;
            if (c == 0.0f && len_sq(v) > len_sq(r)) ie = j;
        }
        ++m;
        ih = ie;
        if (ie == i0) break;
    }
    if (m < 3) return false;
    p.count = m;
    for (int i = 0; i < m; ++i) p.v[i] = ps[hull[i]];
    for (int i = 0; i < m; ++i) {
        V2 edge = sub(p.v[i + 1 < m ? i + 1 : 0], p.v[i]);
        p.n[i] = cross_vs(edge, 1.0f);
        normalize(p.n[i]);
    }
    p.centroid = centroid(p.v, m);
    return true;
}

struct Mass { float mass; V2 center; float I; };

// b2PolygonShape.ComputeMass (b2polygonshape.d:376-459)
static Mass poly_mass(const Poly& p, float density) {
    V2 center = mk(0.0f, 0.0f);
    float area = 0.0f, I = 0.0f;
    V2 s = mk(0.0f, 0.0f);
    for (int i = 0; i < p.count; ++i) s = add(s, p.v[i]);
    float inv = 1.0f / (float)p.count;
    s.x *= inv;
    s.y *= inv;
    const float k_inv3 = 1.0f / 3.0f;
    for (int i = 0; i < p.count; ++i) {
        V2 e1 = sub(p.v[i], s);
        V2 e2 = i + 1 < p.count ? sub(p.v[i + 1], s) : sub(p.v[0], s);
        float D = cross(e1, e2);
        float triangleArea = 0.5f * D;
        area += triangleArea;
        center = add(center, scl(triangleArea * k_inv3, add(e1, e2)));
        float ex1 = e1.x, ey1 = e1.y, ex2 = e2.x, ey2 = e2.y;
        float intx2 = (ex1 * ex1 + ex2 * ex1) + ex2 * ex2;
        float inty2 = (ey1 * ey1 + ey2 * ey1) + ey2 * ey2;
        I += ((0.25f * k_inv3) * D) * (intx2 + inty2);
    }
    Mass m;
    m.mass = density * area;
    float ia = 1.0f / area;
    center.x *= ia;
    center.y *= ia;
    m.center = add(center, s);
    m.I = density * I;
    m.I += m.mass * (dot(m.center, m.center) - dot(center, center));
    return m;
}

// b2CircleShape.ComputeMass (b2circleshape.d:120-127)
static Mass circle_mass(V2 p, float radius, float density) {
    Mass m;
    m.mass = ((density * 3.14159265359f) * radius) * radius;
    m.center = p;
    m.I = m.mass * ((0.5f * radius) * radius + dot(p, p));
    return m;
}

}  // namespace hg
