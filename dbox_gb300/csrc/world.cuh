// Device-side layout of a batch of b2Worlds (structure of arrays over all worlds).
//
// Bodies, fixtures (= broad-phase proxies), joints and contact slots of world w
// occupy contiguous index ranges given by WorldInfo.  Within a world:
//  * bodies are in creation order; the reference's body list (head-inserted,
//    b2world.d:88-96) is the reverse, so list walks run from the last index down;
//  * fixtures are in creation order; with create-only worlds the dynamic-tree
//    proxy id of the k-th proxy is 0 for k = 0 and 2k-1 otherwise
//    (b2dynamictree.d:516-564: each leaf insertion also allocates one parent), so
//    sorting pairs by fixture index equals b2PairLessThan order;
//  * contacts are kept oldest first; the world contact list and every body's
//    edge list are head-inserted (b2contactmanager.d:131-166), so list order is
//    descending slot index.
#pragma once
#include "mlp.cuh"

#include <stdint.h>
#include "dmath.cuh"

namespace dg {

struct WorldInfo {
    int body_start, body_count;
    int fix_start, fix_count;
    int joint_start, joint_count;
    int contact_start, contact_cap;
    int hash_start, hash_cap;      // open-addressing table of contact fixture pairs (power of two)
    int pair_start, pair_cap;      // broad-phase pair buffer
    int bx_start;                  // per-body scratch with one extra entry (body_count + 1)
    int kx_start;                  // per-constraint scratch (contact_cap + joint_count + 2)
    int snap_start;                // TOI sweep snapshots (contact_cap entries)
    int proxy_order;               // 1: fixtures out of proxy-id order, walk them by Ctx.proxy_order
    int pair_block;                // 1: the end-of-Solve pairs come from a block of its own (large world)
    int pad2;
};

struct WorldDyn {
    int contact_count;
    uint32_t flags;                // b2World.m_flags (e_newFixture 1, e_clearForces 4)
    int step_complete;
    float inv_dt0;
    int error;                     // DBOX_ERR_* of the last step (0 = ok)
    int islands;                   // islands solved in the last step
    int toi_events;                // TOI events in the last step
    int pair_total;                // pairs the block pass left for AddPair (large worlds)
    // cumulative work counters (never reset on the device; the host takes differences)
    unsigned long long acc_isl_bodies;   // bodies integrated in islands
    unsigned long long acc_isl_contacts; // contact constraints built
    unsigned long long acc_vsolve;       // contact velocity solves
    unsigned long long acc_psolve;       // contact position solves
    unsigned long long acc_contacts;     // live contacts seen by Collide
    unsigned long long acc_toi_events;
    unsigned long long acc_steps;
    unsigned long long acc_pairs;        // broad-phase pairs emitted
    // solver quality of the last step (measure mode): one extra non-mutating velocity sweep
    // after the last iteration gives |lambda_next - lambda| per contact point (normal and
    // tangent together); the position manifold after the step gives the deepest separation
    float q_sumsq;                 // sum over points of |dlambda|^2
    float q_max;                   // max over points of |dlambda|
    int q_points;                  // points measured
    float q_minsep;                // minimum separation over points after the step (<= 0)
    int ev_count;                  // contact-listener events recorded in the last step
    int ev_pad;
    // the grid of a large world's end-of-solve pair search (k_pairs_block), kept for the pair
    // searches of its SolveTOI events: origin, 1 / cell size, cells per row and column,
    // ordinary and wide proxies, and whether it describes this step's boxes
    float g_ox, g_oy, g_inv;
    int g_ncx, g_ncy, g_nv, g_nwide, g_valid;
    // a large world's Solve on a cluster: what its first block tells the others after the island
    // search (levels, island joints, islands, island bodies and contacts), the count of rows
    // waiting for a prediction, and the continue flag of each position iteration
    int sw_maxv, sw_maxp, sw_njI, sw_go, sw_nisl, sw_nbi, sw_nci, sw_npend;
    // a large world's SolveTOI candidates, counted by its cluster before the event loop
    int toi_ncand, toi_pad;
};

struct BodyStatic {
    float lin_damping, ang_damping, gravity_scale;
    int world;
    int fix_start, fix_count;      // into Ctx.body_fix
    int jadj_start, jadj_count;    // into Ctx.jadj_joint / jadj_other (descending joint index)
};

enum { kRevoluteJoint = 0, kDistanceJoint = 1, kRopeJoint = 2, kWeldJoint = 3, kFrictionJoint = 4, kMotorJoint = 5,
       kWheelJoint = 6, kPrismaticJoint = 7, kPulleyJoint = 8, kMouseJoint = 9, kGearJoint = 10 };
// b2RevoluteJoint / b2DistanceJoint / b2RopeJoint / b2WeldJoint / b2FrictionJoint / b2MotorJoint /
// b2WheelJoint / b2PrismaticJoint / b2PulleyJoint / b2MouseJoint (joints/b2revolutejoint.d,
// b2distancejoint.d, b2ropejoint.d, b2weldjoint.d, b2frictionjoint.d, b2motorjoint.d,
// b2wheeljoint.d, b2prismaticjoint.d, b2pulleyjoint.d, b2mousejoint.d)
struct DJoint {
    int body_a, body_b;
    int collide_connected;
    int island_flag;
    float2 local_anchor_a, local_anchor_b;
    float reference_angle;
    int enable_limit;
    float lower_angle, upper_angle;
    int enable_motor;
    float motor_speed, max_motor_torque;
    float impulse[3];
    float motor_impulse;
    int limit_state;
    float2 rA, rB, lcA, lcB;
    float invMassA, invMassB, invIA, invIB;
    float mass[9];                 // ex.x ex.y ex.z ey.x ey.y ey.z ez.x ez.y ez.z; distance: mass[0]
    float motor_mass;
    int type;                      // k*Joint; distance and rope joints keep their impulse in impulse[0]
    float length, frequency_hz, damping_ratio, gamma, bias;   // distance (length), rope (maximum length), weld
    float2 u;                      // distance / rope: unit vector from anchor A to anchor B
    float cur_length;              // rope: anchor distance at InitVelocityConstraints
    // friction / motor: linear impulse in impulse[0..1], angular in impulse[2]; the linear
    // mass (a b2Mat22) in mass[0] ex.x, mass[1] ex.y, mass[3] ey.x, mass[4] ey.y
    float max_force, max_torque, correction_factor, angular_offset, angular_error, angular_mass;
    float2 linear_offset, linear_error;
    // wheel: point-to-line impulse impulse[0] and mass mass[0], spring impulse impulse[1]
    float2 local_axis_x, local_axis_y, ax, ay;
    float sAx, sBx, sAy, sBy, spring_mass;
    // prismatic: axes in local_axis_x / local_axis_y, impulse[0..2] (perpendicular, angular,
    // limit), K in mass[9], motor as the revolute's fields with max_motor_force
    float lower_translation, upper_translation, max_motor_force;
    float s1, s2, a1, a2;
    float2 axis, perp;
    // pulley: impulse[0], mass[0]; mouse: impulse[0..1], mass matrix as friction's
    float2 ground_a, ground_b, uA, uB, target, mouse_c;
    float ratio, constant, beta;
    float length_a, length_b;      // pulley: the definition's lengths (kept for the dump)
    int pad4;
    // gear (joints/b2gearjoint.d): joint1 joins body_c (its A) to body_a (its B), joint2 body_d
    // to body_b; ratio / constant as the pulley's, the impulse in impulse[0], the mass in mass[0]
    int joint1, joint2, type_a, type_b, body_c, body_d;
    float2 local_anchor_c, local_anchor_d, local_axis_c, local_axis_d, lcC, lcD, jv_ac, jv_bd;
    float reference_angle_a, reference_angle_b, jw_a, jw_b, jw_c, jw_d, invMassC, invMassD, invIC, invID;
};

// b2ContactVelocityConstraint (contacts/b2contactsolver.d:43-58) with body indices in place of island indices.
struct VPoint { float2 rA, rB; float normalImpulse, tangentImpulse, normalMass, tangentMass, velocityBias; };
struct __align__(16) VC {
    VPoint p[2];
    float2 normal;
    float K[4];         // ex.x ex.y ey.x ey.y
    float NM[4];        // normalMass
    int bodyA, bodyB;
    float invMassA, invMassB, invIA, invIB;
    float friction, restitution, tangentSpeed;
    int pointCount;
};
// b2ContactPositionConstraint (b2contactsolver.d:801-814)
struct __align__(16) PC {
    float2 localPoints[2];
    float2 localNormal, localPoint;
    float2 lcA, lcB;
    int bodyA, bodyB;
    float invMassA, invMassB, invIA, invIB;
    int type;
    float radiusA, radiusB;
    int pointCount;
};

// Stored forms of the two constraints, read with 16-byte vector loads.  The solver
// works on VC / PC in registers; these rows hold the same values (the normal mass
// matrices are symmetric, K.ex.y == K.ey.x, so three entries each are kept).
struct __align__(16) VRow {
    float4 r0;          // rA.x rA.y rB.x rB.y of point 0
    float4 r1;          // the same for point 1
    float4 imp;         // normalImpulse0 tangentImpulse0 normalImpulse1 tangentImpulse1
    float4 mass;        // normalMass0 tangentMass0 normalMass1 tangentMass1
    float4 nb;          // normal.x normal.y velocityBias0 velocityBias1
    float4 K;           // K.ex.x K.ex.y K.ey.y friction
    float4 NM;          // normalMass.ex.x .ex.y .ey.y tangentSpeed
    float4 inv;         // invMassA invIA invMassB invIB
    int4 ids;           // bodyA bodyB pointCount item (contact slot, or -1 - joint)
};
struct __align__(16) PRow {
    float4 lp;          // localPoints[0] localPoints[1]
    float4 ln;          // localNormal localPoint
    float4 lc;          // localCenterA localCenterB
    float4 inv;         // invMassA invIA invMassB invIB
    float4 rad;         // radiusA radiusB (z, w unused)
    int4 ids;           // bodyA bodyB meta island; meta = type | pointCount << 4, or -1 - joint
};

// TOI sweep snapshot of one contact's two bodies (taken in list order).
struct SweepSnap { Sweep a, b; float alpha0; int pad; };

constexpr int kProfSlots = 32;         // per-world slots of the optional phase profile
constexpr int kSolveWarps = 4;          // most warp slots (worlds) per block of the solve kernel
constexpr int kStageFloats = 2 * 32 * 36; // per warp: row ring of two 4608-byte halves
constexpr int kWarpSmemFloats = kStageFloats + 4;   // + the ring's two mbarriers

struct Ctx {
    int W;
    int total_bodies, total_fixtures, total_contacts, total_joints;
    const WorldInfo* wi;
    WorldDyn* wd;
    // bodies
    dbox_body_state* bs;
    const BodyStatic* bst;
    const int* body_fix;
    const int* jadj_joint;
    const int* jadj_other;
    // fixtures / proxies
    const DFixture* fx;
    dbox_proxy_state* px;
    // joints
    DJoint* jt;
    // contacts
    dbox_contact_state* ct;
    const int* c_world;            // world of each contact slot
    unsigned long long* hash;      // contact pair table
    int2* pairs;
    // scratch (body-indexed)
    int* s_woken;                  // smallest contact-list position that woke the body this Collide
    int* s_adj_start;              // bx-indexed, body_count+1 per world
    int* s_cursor;                 // body-indexed
    int* s_stack;                  // body-indexed
    int* s_isl_body;               // body-indexed (world-relative positions)
    int* s_body_island;            // body-indexed
    int* s_last;                   // body-indexed
    int* s_isl_bstart;             // bx-indexed: island -> start in s_isl_body
    int* s_isl_cstart;             // bx-indexed
    int* s_isl_jstart;             // bx-indexed
    unsigned* s_isl_minsep;        // body-indexed (island id), ordered-float key
    int* s_isl_flags;              // body-indexed (island id): bit0 done, bit1 solved, bit2 joints not ok
    unsigned* s_isl_sleep;         // body-indexed (island id)
    int* s_pcount;                 // fixture-indexed: pair counts / moved list
    int* s_moved;                  // fixture-indexed
    unsigned* s_sapk[2];           // fixture-indexed: sweep-and-prune keys (radix-sort ping-pong)
    int* s_sapi[2];                // fixture-indexed: proxy of each sorted key (top bit: moved)
    float4* s_sapbox;              // fixture-indexed: fat AABBs in sorted order
    int* s_sapcell;                // per world 8 * fixtures + 130 from 8 * fix_start + 130 * world: cell tables
    const int* big_worlds;         // the worlds whose end-of-Solve pairs a block generates
    int n_big;
    int big_block;                 // 1: large worlds run b2World.Solve on a block (k_solve_big), not a warp
    int big_cluster;               // blocks per large world in k_solve_big's level sweeps (a thread-block cluster)
    int steps;                     // steps each world takes in one launch of k_step_fused
    const int* proxy_order;        // fixture-indexed: world-local fixture of each proxy-id rank
    // scratch (contact-indexed)
    int* s_cstate;                 // 0 processed, 1 inactive, 2 destroyed
    int2* s_adj_items;             // 2 per contact slot: (contact, other body) edges by body
    int2* s_isl_pair;              // contact-slot-indexed: bodies of the island contact sequence
    int* s_tcand;                  // contact-slot-indexed: TOI candidate contacts of the world
    int* s_isl_contact;            // contact-slot-indexed
    int* s_level;                  // kx-indexed
    int* s_sched_v;                // kx-indexed
    int* s_lvl_v;                  // kx-indexed (+1)
    int* s_sched_p;
    int* s_lvl_p;
    int* s_tmp;                    // kx-indexed sequence-order items while sorting by level
    int* s_lcur;                   // kx-indexed level cursors while bucketing by level
    int* s_isl_joint;              // joint-indexed
    int* s_accept;                 // pair-indexed
    VRow* vr;                      // kx-indexed: velocity rows in velocity-schedule order
    PRow* pr;                      // kx-indexed: position rows in position-schedule order
    VRow* tvr;                     // 32 per world: rows of the current TOI island
    PRow* tpr;                     // 32 per world
    int* s_vpos;                   // contact-slot-indexed: velocity-schedule position (worlds with joints)
    const int* solve_world;        // per warp slot of the solve kernel: world index or -1
    const int* solve_smem;         // per warp slot: float offset of its body rows in shared memory, or -1
    int solve_blocks;              // blocks of the solve kernel
    int solve_wpb;                 // warp slots per block (1, 2 or kSolveWarps)
    int solve_smem_floats;         // dynamic shared memory of one solve block, in floats
    // world-queue mapping (solve_queue != nullptr): one resident wave of warps takes worlds
    // from solve_order (costliest first); the first solve_heavy entries go one per SM
    // sub-partition at a time
    const int* solve_order;        // W world indices, costliest first
    int* solve_queue;              // [0] next heavy entry, [1] next light entry, [2 + 4*sm + sub] heavy flags
    int solve_heavy;               // number of heavy entries at the front of solve_order
    int solve_exclusive;           // a warp whose sub-partition runs a heavy world takes no light world meanwhile
    int solve_cap;                 // bodies per warp region of shared memory (larger worlds use global rows)
    int solve_nsm;                 // SMs of the device
    SweepSnap* snap;               // contact-slot-indexed
    int2* s_cbody;                 // contact-slot-indexed: world-local bodies of the contact
    unsigned char* s_cq;           // contact-slot-indexed: bit0 island-graph edge, bit1 sensor
    unsigned char* s_cvis;         // contact-slot-indexed: visited by the island search
    unsigned char* s_bfl;          // body-indexed: awake/active/static/dynamic/visited/mark bits
    float* s_sbody;                // 6 per body: solver velocity and position (global fallback)
    // step parameters
    float dt, inv_dt;
    int vel_iters, pos_iters;
    float2 gravity;
    int warm_starting, continuous, sub_stepping, allow_sleep;
    int record_events;
    dbox_contact_event* events;    // per world: 4 * contact_start + 64 * world, 4 * contact_cap + 64 records
    unsigned char* s_cevt;         // contact-slot-indexed: listener events of this Collide (1 begin, 2 end, 4 presolve)
    int* g_status;                 // bit (-code) set for every DBOX_ERR_* raised by any world
    // learned warm start: 0 plain (Box2D), 1 plain + log training samples, 2 learned start
    int ws_mode;
    MlpDev mlp;                    // ws_mode 2: the network
    const dbox_contact_state* start_ct;  // ws_mode 3: contacts (same slots) whose impulses start the new points
    float* samples;                // ws_mode 1: kSampleFloats per sample (32 features, 4 targets)
    unsigned* sample_count;        // ws_mode 1: samples written so far (may exceed sample_cap)
    int sample_cap;
    int* s_slog;                   // kx-indexed: sample slot of the velocity row, or -1
    float* s_feat;                 // contact-slot-indexed: 32 features per pending learned contact
    int* s_pend;                   // contact-slot-indexed: velocity-schedule positions awaiting a prediction
    int measure;                   // 1: fill the q_* fields of WorldDyn each step
    int wait_polls;                // polls an mbarrier wait may take before it counts as DBOX_ERR_TIMEOUT
    const int* fmode;              // per world: 0 the default contact filter, 1 table and default, 2 table only
    const unsigned long long* ftab;  // per world 64 rows: class a collides with class b when bit b of row a is set
    float* s_vsave;                // body-indexed, 3 floats: velocities kept across the measuring sweep
    unsigned long long* prof;      // optional: kProfSlots clock64 figures per world (NULL = off)
};

// ------------------------------------------------------------ body state helpers (dbox_body_state fields)
DG int btype(const dbox_body_state& b) { return b.type; }
DG float2 b_c(const dbox_body_state& b) { return v2(b.sweep[4], b.sweep[5]); }
DG float2 b_lc(const dbox_body_state& b) { return v2(b.sweep[0], b.sweep[1]); }
DG float2 b_v(const dbox_body_state& b) { return v2(b.vel[0], b.vel[1]); }
DG Xf b_xf(const dbox_body_state& b) { Xf x; x.p = v2(b.xf[0], b.xf[1]); x.q.s = b.xf[2]; x.q.c = b.xf[3]; return x; }
DG Sweep b_sweep(const dbox_body_state& b) {
    Sweep s;
    s.lc = v2(b.sweep[0], b.sweep[1]);
    s.c0 = v2(b.sweep[2], b.sweep[3]);
    s.c = v2(b.sweep[4], b.sweep[5]);
    s.a0 = b.sweep[6];
    s.a = b.sweep[7];
    s.alpha0 = b.sweep[8];
    return s;
}
DG void b_set_sweep(dbox_body_state& b, const Sweep& s) {
    b.sweep[0] = s.lc.x; b.sweep[1] = s.lc.y;
    b.sweep[2] = s.c0.x; b.sweep[3] = s.c0.y;
    b.sweep[4] = s.c.x; b.sweep[5] = s.c.y;
    b.sweep[6] = s.a0; b.sweep[7] = s.a; b.sweep[8] = s.alpha0;
}
// b2Body.SynchronizeTransform (b2body.d:1143-1147)
DG void b_sync_transform(dbox_body_state& b) {
    Rot q = rot(b.sweep[7]);
    float2 p = v2(b.sweep[4], b.sweep[5]) - mul(q, v2(b.sweep[0], b.sweep[1]));
    b.xf[0] = p.x; b.xf[1] = p.y; b.xf[2] = q.s; b.xf[3] = q.c;
}
// b2Body.SetAwake (b2body.d:827-846)
DG void b_set_awake(dbox_body_state& b, bool flag) {
    if (flag) {
        if ((b.flags & kBodyAwake) == 0) { b.flags |= kBodyAwake; b.sleep_time = 0.0f; }
    } else {
        b.flags &= ~(uint32_t)kBodyAwake;
        b.sleep_time = 0.0f;
        b.vel[0] = 0.0f; b.vel[1] = 0.0f; b.vel[2] = 0.0f;
        b.force[0] = 0.0f; b.force[1] = 0.0f; b.force[2] = 0.0f;
    }
}
// b2Body.Advance (b2body.d:1172-1180)
DG void b_advance(dbox_body_state& b, float alpha) {
    Sweep s = b_sweep(b);
    sweep_advance(s, alpha);
    s.c = s.c0;
    s.a = s.a0;
    b_set_sweep(b, s);
    Rot q = rot(s.a);
    float2 p = s.c - mul(q, s.lc);
    b.xf[0] = p.x; b.xf[1] = p.y; b.xf[2] = q.s; b.xf[3] = q.c;
}

// ordered key of a float for unsigned atomicMin
DG unsigned fkey(float f) {
    unsigned u = __float_as_uint(f);
    return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}
DG float funkey(unsigned k) {
    unsigned u = (k & 0x80000000u) ? (k & 0x7fffffffu) : ~k;
    return __uint_as_float(u);
}

DG void set_error(const Ctx& x, int w, int code) {
    atomicCAS(&x.wd[w].error, 0, code);
    atomicOr(x.g_status, 1 << (-code));
}

}  // namespace dg

// Device arrays of the world-query index (query.cu), filled by the host (api.cu).
struct dbox_query_buffers {
    int W;
    const dg::WorldInfo* wi;
    const dg::DFixture* fx;
    const dbox_proxy_state* px;
    const dbox_body_state* bs;
    float4* box;
    int* idx;
    float4* bucket;
    float4* group;
    int* live;
    unsigned* key0;
    unsigned* key1;
    int* sidx0;
    int* sidx1;
    unsigned* bitmap;
    int bm_words;
    int query_blocks;
};

