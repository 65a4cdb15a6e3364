/*
 * dbox_gpu.h - C ABI of the GB300 b2World.Step library (libdbox_gpu.so).
 *
 * Drop-in boundary for the per-step hot path of dbox (a D port of Box2D 2.3.1).
 * Every entry point is plain C: int32 status return (0 = ok, negative =
 * DBOX_ERR_*), plain pointers and sizes, no exceptions, no torch types.
 * Each declaration names the reference interface it replaces (paths are within
 * the dbox project, src/dbox/...).
 *
 * Ownership: the library owns all device memory of a world; host buffers passed
 * in are caller-owned and copied.  A world is not reentrant: one thread at a time.
 *
 * A "world" handle holds one or more independent simulation worlds stored
 * side by side on the GPU (a batch).  The single-world calls address world 0.
 */
#ifndef DBOX_GPU_H
#define DBOX_GPU_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---------------------------------------------------------------- status */
#define DBOX_OK 0
#define DBOX_ERR_INVALID -1    /* bad argument (null pointer, index out of range, bad count) */
#define DBOX_ERR_LOCKED -2     /* call not allowed while the world is stepping (b2World.IsLocked) */
#define DBOX_ERR_CAPACITY -3   /* a device pool (contacts, pairs, islands) overflowed */
#define DBOX_ERR_TIMEOUT -4    /* a bounded device loop hit its iteration limit */
#define DBOX_ERR_NAN -5        /* non-finite body state after a step */
#define DBOX_ERR_CUDA -6       /* a CUDA runtime call failed; see dbox_last_error() */
#define DBOX_ERR_UNSUPPORTED -7 /* feature outside the implemented path (e.g. edge shapes) */

/* ---------------------------------------------------------------- types */
typedef struct { float x, y; } dbox_vec2;
/* b2AABB (collision/b2collision.d:300-345) */
typedef struct { dbox_vec2 lower, upper; } dbox_aabb;
/* One ray hit: the fixture, b2RayCastOutput.fraction, the point (1 - fraction) p1 + fraction p2
 * and b2RayCastOutput.normal, as b2WorldRayCastWrapper hands them to ReportFixture
 * (dynamics/b2world.d:1605-1629). */
typedef struct { int32_t fixture; float fraction; dbox_vec2 point, normal; } dbox_ray_hit;

/* b2BodyType (dynamics/b2body.d:34-42) */
#define DBOX_STATIC_BODY 0
#define DBOX_KINEMATIC_BODY 1
#define DBOX_DYNAMIC_BODY 2

/* b2BodyDef (dynamics/b2body.d:51-104); dbox_body_def_default() gives the reference defaults. */
typedef struct {
    int32_t type;
    dbox_vec2 position;
    float angle;
    dbox_vec2 linear_velocity;
    float angular_velocity;
    float linear_damping;
    float angular_damping;
    int32_t allow_sleep;
    int32_t awake;
    int32_t fixed_rotation;
    int32_t bullet;
    int32_t active;
    float gravity_scale;
} dbox_body_def;

/* Shape kinds accepted by fixture creation. */
#define DBOX_SHAPE_CIRCLE 0      /* b2CircleShape: m_p = center, m_radius = radius */
#define DBOX_SHAPE_POLYGON 1     /* b2PolygonShape.Set(vertices, count): weld + gift-wrap hull */
#define DBOX_SHAPE_BOX 2         /* b2PolygonShape.SetAsBox(hx, hy) */
#define DBOX_SHAPE_ORIENTED_BOX 3 /* b2PolygonShape.SetAsBox(hx, hy, center, angle) */
#define DBOX_SHAPE_EDGE 4        /* b2EdgeShape: vertices[0..1] = vertex1, vertex2; count bit 0 =
                                    hasVertex0 with vertices[2] = vertex0, bit 1 = hasVertex3 with
                                    vertices[3] = vertex3 (the neighbours for smooth collision) */

typedef struct {
    int32_t kind;            /* DBOX_SHAPE_* */
    int32_t count;           /* POLYGON: number of input points (3..8) */
    dbox_vec2 vertices[8];   /* POLYGON input points */
    dbox_vec2 center;        /* CIRCLE: center; ORIENTED_BOX: box center */
    float radius;            /* CIRCLE radius */
    float hx, hy;            /* BOX / ORIENTED_BOX half extents */
    float angle;             /* ORIENTED_BOX angle */
} dbox_shape_def;

/* b2FixtureDef + b2Filter (dynamics/b2fixture.d:32-73) */
typedef struct {
    float friction;          /* default 0.2 */
    float restitution;
    float density;
    int32_t is_sensor;
    uint16_t category_bits;  /* default 0x0001 */
    uint16_t mask_bits;      /* default 0xFFFF */
    int16_t group_index;
    int16_t pad_;
} dbox_fixture_def;

/* b2RevoluteJointDef (dynamics/joints/b2revolutejoint.d:30-110) */
typedef struct {
    int32_t body_a, body_b;
    int32_t collide_connected;
    dbox_vec2 local_anchor_a, local_anchor_b;
    float reference_angle;
    int32_t enable_limit;
    float lower_angle, upper_angle;
    int32_t enable_motor;
    float motor_speed, max_motor_torque;
} dbox_revolute_def;

/* b2DistanceJointDef (dynamics/joints/b2distancejoint.d:33-93) */
typedef struct {
    int32_t body_a, body_b;
    int32_t collide_connected;
    dbox_vec2 local_anchor_a, local_anchor_b;
    float length;          /* natural length between the anchors */
    float frequency_hz;    /* mass-spring-damper frequency; 0 = rigid */
    float damping_ratio;
} dbox_distance_def;

/* b2RopeJointDef (dynamics/joints/b2ropejoint.d:30-52) */
typedef struct {
    int32_t body_a, body_b;
    int32_t collide_connected;
    dbox_vec2 local_anchor_a, local_anchor_b;
    float max_length;
} dbox_rope_def;

/* b2WeldJointDef (dynamics/joints/b2weldjoint.d:30-86) */
typedef struct {
    int32_t body_a, body_b;
    int32_t collide_connected;
    dbox_vec2 local_anchor_a, local_anchor_b;
    float reference_angle;
    float frequency_hz;    /* angular softness; 0 = rigid */
    float damping_ratio;
} dbox_weld_def;

/* b2FrictionJointDef (dynamics/joints/b2frictionjoint.d:30-73) */
typedef struct {
    int32_t body_a, body_b;
    int32_t collide_connected;
    dbox_vec2 local_anchor_a, local_anchor_b;
    float max_force, max_torque;
} dbox_friction_def;

/* b2MotorJointDef (dynamics/joints/b2motorjoint.d:30-80) */
typedef struct {
    int32_t body_a, body_b;
    int32_t collide_connected;
    dbox_vec2 linear_offset;     /* position of body B minus the position of body A, in A's frame */
    float angular_offset;        /* angle of body B minus the angle of body A */
    float max_force, max_torque;
    float correction_factor;     /* position correction factor in [0, 1] */
} dbox_motor_def;

/* b2WheelJointDef (dynamics/joints/b2wheeljoint.d:30-99) */
typedef struct {
    int32_t body_a, body_b;
    int32_t collide_connected;
    dbox_vec2 local_anchor_a, local_anchor_b;
    dbox_vec2 local_axis_a;      /* translation axis in body A (unit length) */
    int32_t enable_motor;
    float max_motor_torque, motor_speed;
    float frequency_hz, damping_ratio;   /* suspension spring */
} dbox_wheel_def;

/* b2PrismaticJointDef (dynamics/joints/b2prismaticjoint.d:30-158) */
typedef struct {
    int32_t body_a, body_b;
    int32_t collide_connected;
    dbox_vec2 local_anchor_a, local_anchor_b;
    dbox_vec2 local_axis_a;      /* translation axis in body A (normalised on creation) */
    float reference_angle;
    int32_t enable_limit;
    float lower_translation, upper_translation;
    int32_t enable_motor;
    float max_motor_force, motor_speed;
} dbox_prismatic_def;

/* b2PulleyJointDef (dynamics/joints/b2pulleyjoint.d:30-97) */
typedef struct {
    int32_t body_a, body_b;
    int32_t collide_connected;
    dbox_vec2 ground_anchor_a, ground_anchor_b;   /* world points the two sides hang from */
    dbox_vec2 local_anchor_a, local_anchor_b;
    float length_a, length_b;                     /* reference lengths of the two sides */
    float ratio;                                  /* lengthA + ratio * lengthB stays constant */
} dbox_pulley_def;

/* b2MouseJointDef (dynamics/joints/b2mousejoint.d:28-58): drags body_b's point under
 * `target` towards the target; body_a only anchors the joint (usually the ground). */
typedef struct {
    int32_t body_a, body_b;
    int32_t collide_connected;
    dbox_vec2 target;
    float max_force, frequency_hz, damping_ratio;
} dbox_mouse_def;

/* b2GearJointDef (dynamics/joints/b2gearjoint.d:30-48): couples joint1 and joint2, each a
 * revolute or prismatic joint; the gear acts on joint1's body B, joint2's body B and, through
 * them, on the joints' A bodies.  body_a / body_b are the definition's bodies, which the
 * reference uses only to flag their contacts for filtering (b2world.d:236-254). */
typedef struct {
    int32_t body_a, body_b;
    int32_t collide_connected;
    int32_t joint1, joint2;
    float ratio;
} dbox_gear_def;

/* ------------------------------------------------------- world snapshot
 * Flat state records, used by dbox_world_export_state / import_state
 * (exact checkpoint/resume) and by the parity tests.  Flag words use the
 * reference's bit values (b2Body e_* b2body.d:1118-1127, b2Contact e_*
 * contacts/b2contact.d:242-261, b2World e_* b2world.d:922-927). */
typedef struct {
    int32_t body_count, fixture_count, contact_count, joint_count;
    uint32_t world_flags;     /* e_newFixture 1, e_locked 2, e_clearForces 4 */
    int32_t step_complete;    /* b2World.m_stepComplete */
    float inv_dt0;            /* b2World.m_inv_dt0 */
    int32_t reserved;
} dbox_world_header;

typedef struct {
    uint32_t flags;          /* island 1, awake 2, autoSleep 4, bullet 8, fixedRotation 0x10, active 0x20 */
    int32_t type;
    float xf[4];             /* p.x, p.y, q.s, q.c */
    float sweep[9];          /* localCenter.x/y, c0.x/y, c.x/y, a0, a, alpha0 */
    float vel[3];            /* v.x, v.y, w */
    float force[3];          /* force.x, force.y, torque */
    float sleep_time;
    float mass[4];           /* mass, invMass, I, invI */
} dbox_body_state;

typedef struct {
    float fat_aabb[4];       /* lowerBound.x/y, upperBound.x/y of the dynamic-tree leaf */
    int32_t moved;           /* 1 if the proxy is in the broad-phase move buffer */
    int32_t proxy_id;        /* dynamic-tree node id of the proxy */
} dbox_proxy_state;

typedef struct {
    float local_point[2];
    float normal_impulse, tangent_impulse;
    uint32_t id;             /* b2ContactID.key: indexA | indexB<<8 | typeA<<16 | typeB<<24 */
} dbox_manifold_point;

typedef struct {
    int32_t fixture_a, fixture_b;  /* fixture creation indices, after the type-order swap */
    uint32_t flags;                /* island 1, touching 2, enabled 4, filter 8, bulletHit 0x10, toi 0x20 */
    int32_t toi_count;
    float toi, friction, restitution, tangent_speed;
    int32_t point_count, type;     /* b2Manifold.pointCount / type (circles 0, faceA 1, faceB 2) */
    float local_normal[2], local_point[2];
    dbox_manifold_point points[2];
} dbox_contact_state;              /* exported oldest first = reverse of b2World.GetContactList order */

typedef struct {
    float impulse[3];
    float motor_impulse;
    int32_t limit_state;
} dbox_joint_state;

/* b2Profile (dynamics/b2timestep.d:37-47), milliseconds, measured with CUDA events. */
typedef struct {
    float step, collide, solve, solve_init, solve_velocity, solve_position, broadphase, solve_toi;
} dbox_profile;

/* Contact listener (b2ContactListener, dynamics/b2worldcallbacks.d:87-128).
 * Events are recorded on the device in reference order and delivered on the
 * calling thread before dbox_world_step returns. */
#define DBOX_EVENT_BEGIN 1
#define DBOX_EVENT_END 2
#define DBOX_EVENT_PRESOLVE 3
#define DBOX_EVENT_POSTSOLVE 4
typedef struct {
    int32_t kind;              /* DBOX_EVENT_* */
    int32_t world;             /* world index inside the handle */
    int32_t fixture_a, fixture_b;
    int32_t point_count;       /* manifold points (BEGIN/PRESOLVE) or impulse count (POSTSOLVE) */
    float normal_impulses[2];
    float tangent_impulses[2];
} dbox_contact_event;
typedef void (*dbox_event_fn)(const dbox_contact_event* events, int32_t count, void* user);

typedef struct dbox_world dbox_world;

/* -------------------------------------------------------------- lifecycle */

/* Sizing hints; zero fields take defaults. */
typedef struct {
    int32_t contacts_per_body;   /* contact pool per world = contacts_per_body * bodies + 64 (default 8) */
    int32_t team;                /* 0 auto, 32 = one warp per world, 128/256/512 = one block per world */
} dbox_world_caps;

/* b2World(gravity) constructor (dynamics/b2world.d:865-895). Creates n_worlds
 * independent worlds sharing gravity; worlds are addressed 0..n_worlds-1. */
int32_t dbox_world_create(dbox_vec2 gravity, int32_t n_worlds, const dbox_world_caps* caps,
                          dbox_world** out);
/* b2World destructor (b2world.d:897-920). */
int32_t dbox_world_destroy(dbox_world* w);

/* Fill reference defaults (b2BodyDef b2body.d:51-104, b2FixtureDef b2fixture.d:49-73). */
void dbox_body_def_default(dbox_body_def* def);
void dbox_fixture_def_default(dbox_fixture_def* def);

/* b2World.CreateBody (b2world.d:75-99). Body ids count from 0 per world, in creation order. */
int32_t dbox_body_create(dbox_world* w, int32_t world, const dbox_body_def* def, int32_t* out_body);
/* b2Body.CreateFixture(def) (b2body.d:116-155) with the shape of b2PolygonShape.Set/SetAsBox
 * (collision/shapes/b2polygonshape.d:74-262) or b2CircleShape (b2circleshape.d). */
int32_t dbox_fixture_create(dbox_world* w, int32_t world, int32_t body, const dbox_shape_def* shape,
                            const dbox_fixture_def* def, int32_t* out_fixture);
/* b2Body.CreateFixture with a b2ChainShape (collision/shapes/b2chainshape.d): CreateChain(vertices,
 * count) or, with loop != 0, CreateLoop; prev / next (may be NULL) are SetPrevVertex /
 * SetNextVertex.  The chain is created as its child edges (b2ChainShape.GetChildEdge), one
 * fixture index per child in child order, each with the chain's neighbour vertices as ghost
 * vertices: the same proxies (ids in child order), pairs, contacts (a chain child first, no
 * chain-edge or chain-chain contacts) and manifolds as the reference's chain.  A chain has no
 * mass; its child edges are created with density 0.  out_first receives the first child's
 * fixture index. */
int32_t dbox_fixture_create_chain(dbox_world* w, int32_t world, int32_t body, const dbox_vec2* vertices, int32_t count,
                                  int32_t loop, const dbox_vec2* prev_vertex, const dbox_vec2* next_vertex,
                                  const dbox_fixture_def* def, int32_t* out_first);
/* b2World.DestroyBody (dynamics/b2world.d:105-193): its joints (newest first), its contacts
 * (EndContact to the listener for touching ones, waking both bodies of contacts with points),
 * then its fixtures' broad-phase proxies.  b2Body.DestroyFixture (dynamics/b2body.d:179-247):
 * the fixture's contacts, its proxies, then the body's mass (a chain child destroys its whole
 * chain, as the reference's chain fixture).  b2World.DestroyJoint (dynamics/b2world.d:265-360):
 * wakes both bodies and flags their contacts for filtering unless collideConnected.  Between
 * steps only.  Indices of other bodies, fixtures and joints do not change; a destroyed one
 * exports as an all-zero record (a proxy of id -1).  New proxies take the ids the reference's
 * tree hands out: freed leaves last in, first out, then never-used node ids.  Destroying one
 * of a gear joint's own bodies (its joint1's or joint2's body B) destroys the gear first, as the
 * reference's newest-first joint walk does.  A joint a gear uses, or a body that carries such a
 * joint but is neither of the gear's own bodies, cannot be destroyed before the gear
 * (DBOX_ERR_INVALID): the reference would leave the gear holding a destroyed joint. */
int32_t dbox_body_destroy(dbox_world* w, int32_t world, int32_t body);
/* b2World.CreateJoint with a b2GearJointDef (joints/b2gearjoint.d:83-168): joint1 and joint2
 * are live revolute or prismatic joints of the same world; a joint a gear uses cannot be
 * destroyed before the gear (DBOX_ERR_INVALID). */
int32_t dbox_joint_create_gear(dbox_world* w, int32_t world, const dbox_gear_def* def, int32_t* out_joint);
int32_t dbox_fixture_destroy(dbox_world* w, int32_t world, int32_t fixture);
int32_t dbox_joint_destroy(dbox_world* w, int32_t world, int32_t joint);

/* b2World.CreateJoint with a b2RevoluteJointDef (b2world.d:196-261, joints/b2revolutejoint.d). */
int32_t dbox_joint_create_revolute(dbox_world* w, int32_t world, const dbox_revolute_def* def,
                                   int32_t* out_joint);
/* b2World.CreateJoint with a b2DistanceJointDef (b2world.d:196-261, joints/b2distancejoint.d).
 * Joint indices count all joint kinds in creation order; the snapshot's impulse[0] holds the
 * distance joint's impulse. */
int32_t dbox_joint_create_distance(dbox_world* w, int32_t world, const dbox_distance_def* def,
                                   int32_t* out_joint);
/* b2World.CreateJoint with a b2RopeJointDef (joints/b2ropejoint.d); snapshot: impulse[0], limit_state. */
int32_t dbox_joint_create_rope(dbox_world* w, int32_t world, const dbox_rope_def* def, int32_t* out_joint);
/* b2World.CreateJoint with a b2WeldJointDef (joints/b2weldjoint.d); snapshot: impulse[0..2]. */
int32_t dbox_joint_create_weld(dbox_world* w, int32_t world, const dbox_weld_def* def, int32_t* out_joint);
/* b2World.CreateJoint with a b2FrictionJointDef / b2MotorJointDef (joints/b2frictionjoint.d,
 * b2motorjoint.d); snapshot: impulse[0..1] the linear impulse, impulse[2] the angular one. */
int32_t dbox_joint_create_friction(dbox_world* w, int32_t world, const dbox_friction_def* def, int32_t* out_joint);
int32_t dbox_joint_create_motor(dbox_world* w, int32_t world, const dbox_motor_def* def, int32_t* out_joint);
/* b2World.CreateJoint with a b2WheelJointDef (joints/b2wheeljoint.d); snapshot: impulse[0] the
 * point-to-line impulse, impulse[1] the spring impulse, motor_impulse. */
int32_t dbox_joint_create_wheel(dbox_world* w, int32_t world, const dbox_wheel_def* def, int32_t* out_joint);
/* b2World.CreateJoint with a b2PrismaticJointDef (joints/b2prismaticjoint.d); snapshot:
 * impulse[0..2] (perpendicular, angular, limit), motor_impulse, limit_state. */
int32_t dbox_joint_create_prismatic(dbox_world* w, int32_t world, const dbox_prismatic_def* def, int32_t* out_joint);
/* b2World.CreateJoint with a b2PulleyJointDef / b2MouseJointDef (joints/b2pulleyjoint.d,
 * b2mousejoint.d); snapshot: impulse[0] (pulley), impulse[0..1] (mouse).  The mouse joint's
 * local anchor is the target in body B's frame at creation. */
int32_t dbox_joint_create_pulley(dbox_world* w, int32_t world, const dbox_pulley_def* def, int32_t* out_joint);
int32_t dbox_joint_create_mouse(dbox_world* w, int32_t world, const dbox_mouse_def* def, int32_t* out_joint);
/* b2MouseJoint.SetTarget (b2mousejoint.d:83-91): wakes body B and moves the target. */
int32_t dbox_joint_set_mouse_target(dbox_world* w, int32_t world, int32_t joint, dbox_vec2 target);

/* Bulk creation of a whole scene into one world: n bodies, then m fixtures
 * (fixture_body[i] indexes the bodies created by this call), then k joints
 * (body indices relative to this call).  Same effect as the single calls in
 * the order bodies, fixtures, joints. */
int32_t dbox_scene_create(dbox_world* w, int32_t world, int32_t n_bodies, const dbox_body_def* bodies,
                          int32_t n_fixtures, const int32_t* fixture_body, const dbox_shape_def* shapes,
                          const dbox_fixture_def* fixtures, int32_t n_joints, const dbox_revolute_def* joints);

/* World flag setters (b2World.SetWarmStarting/SetContinuousPhysics/SetSubStepping/
 * SetAllowSleeping/SetAutoClearForces, b2world.d:622-753), applied to every world of the handle. */
int32_t dbox_world_set_flags(dbox_world* w, int32_t warm_starting, int32_t continuous,
                             int32_t sub_stepping, int32_t allow_sleep, int32_t auto_clear_forces);
/* b2World.SetGravity (b2world.d:711-714). */
int32_t dbox_world_set_gravity(dbox_world* w, dbox_vec2 gravity);

/* b2World.SetContactListener (b2world.d:59-62): events are delivered through fn,
 * in reference order, at the end of each step.  fn = NULL removes the listener. */
int32_t dbox_world_set_listener(dbox_world* w, dbox_event_fn fn, void* user);

/* b2Fixture.SetFilterData (dynamics/b2fixture.d:132-137): new category, mask and group bits, then
 * b2Fixture.Refilter (:140-180): the fixture's contacts are flagged so that the next Collide
 * checks b2ContactFilter.ShouldCollide again (and destroys those that fail), and its proxies go
 * into the move buffer so that the next FindNewContacts may create new pairs.  Between steps. */
int32_t dbox_fixture_set_filter(dbox_world* w, int32_t world, int32_t fixture, uint16_t category_bits,
                                uint16_t mask_bits, int16_t group_index);
/* b2World.SetContactFilter (dynamics/b2world.d:52-55) with a user b2ContactFilter
 * (b2worldcallbacks.d:47-64) given as data, since ShouldCollide is called on the device (in
 * AddPair, b2contactmanager.d:52-176, and in Collide for flagged contacts, :266-288): every
 * fixture has a filter class 0..63 (0 unless set), and fixtures of classes a and b may collide
 * when bit b of table[a] is set (table: 64 rows, symmetric, else DBOX_ERR_INVALID).  With
 * with_default != 0 the reference's default rule (groups, categories and masks) must pass too, as
 * in a subclass that calls the base class first; with 0 the table alone decides.  table = NULL
 * restores the default filter.  As in the reference, existing contacts are checked again only
 * once flagged (dbox_fixture_set_filter / _class, or joint creation and destruction).
 * dbox_fixture_set_filter_class sets a fixture's class (a chain's children together) and
 * refilters it as dbox_fixture_set_filter does. */
int32_t dbox_world_set_contact_filter(dbox_world* w, int32_t world, const uint64_t* table, int32_t with_default);
int32_t dbox_fixture_set_filter_class(dbox_world* w, int32_t world, int32_t fixture, int32_t filter_class);

/* One b2ContactListener.PreSolve call (dynamics/b2worldcallbacks.d:101-115), made by
 * b2Contact.Update (contacts/b2contact.d:354) for a touching, non-sensor contact during the
 * step's Collide.  `contact` is the contact after its update (fixtures as world-local indices,
 * flags, the new manifold with its warm-start impulses); the old manifold is not passed.  The
 * callback may change the four edit fields, as b2Contact.SetEnabled / SetFriction /
 * SetRestitution / SetTangentSpeed (contacts/b2contact.d:105-190) would: `enabled` 0 disables
 * the contact for this step, the other three persist until changed again. */
typedef struct {
    int32_t world;
    int32_t enabled;               /* in: 1; out: 0 = SetEnabled(false) */
    float friction;                /* in: the contact's friction; out: SetFriction */
    float restitution;             /* in / out: SetRestitution */
    float tangent_speed;           /* in / out: SetTangentSpeed */
    dbox_contact_state contact;    /* read only */
} dbox_presolve_contact;
typedef void (*dbox_presolve_fn)(dbox_presolve_contact* contacts, int32_t count, void* user);

/* b2World.SetContactListener with a PreSolve callback (b2world.d:59-62): while fn is set,
 * every step stops after Collide, hands fn the step's PreSolve calls of all worlds (world by
 * world, each in the reference's order: the contact list walked newest first), applies the
 * edits fn made, then runs the solve.  The edits take effect exactly as in the reference, since
 * a PreSolve edit only touches its own contact and nothing later in Collide reads it.  One
 * difference: b2World.SolveTOI also calls b2Contact.Update (and PreSolve) on the contacts it
 * moves to a time of impact, those with a static, kinematic or bullet body
 * (b2world.d:1194-1208, 1287, 1345-1372); there the library keeps the window's decisions (a
 * contact disabled in the window stays disabled through the step's sub-steps; a contact that
 * first touches inside a sub-step gets no PreSolve call and so no edit) and reports those
 * calls only as recorded PRESOLVE events to the listener of dbox_world_set_listener.  Edits of
 * contacts between dynamic, non-bullet bodies therefore match the reference exactly; edits of
 * contacts with a static, kinematic or bullet body match unless such a contact first touches
 * during a step's time-of-impact sub-steps.  fn = NULL removes it.
 * The window costs one device synchronisation and a download of the affected worlds'
 * contacts per step. */
int32_t dbox_world_set_presolve(dbox_world* w, dbox_presolve_fn fn, void* user);

/* b2World.Step(dt, velocityIterations, positionIterations) (b2world.d:367-434),
 * applied to every world of the handle.  Inputs and outputs stay on the device. */
int32_t dbox_world_step(dbox_world* w, float dt, int32_t velocity_iterations, int32_t position_iterations);

/* Same as dbox_world_step, with `steps` steps captured once into a CUDA graph and replayed. */
int32_t dbox_world_step_n(dbox_world* w, float dt, int32_t velocity_iterations,
                          int32_t position_iterations, int32_t steps);

/* Body readback (b2Body.GetPosition/GetAngle/GetLinearVelocity/GetAngularVelocity,
 * b2body.d:271-340) for every body of every world, in (world, body id) order.
 * Any pointer may be NULL; each non-NULL array holds total_bodies entries. */
int32_t dbox_world_get_bodies(dbox_world* w, dbox_vec2* position, float* angle,
                              dbox_vec2* linear_velocity, float* angular_velocity, int32_t* awake);
/* Body slots of world `world` (body ids run 0 .. count - 1; destroyed bodies keep their slot). */
int32_t dbox_world_body_count(dbox_world* w, int32_t world, int32_t* out);
/* b2World.GetContactCount (b2world.d:695-699). */
int32_t dbox_world_contact_count(dbox_world* w, int32_t world, int32_t* out);
/* b2World.GetBodyCount / GetJointCount / GetContactCount (b2world.d:683-699): live bodies and
 * joints (destroyed ones not counted) and contacts of world `world`; any pointer may be NULL. */
int32_t dbox_world_get_counts(dbox_world* w, int32_t world, int32_t* bodies, int32_t* joints, int32_t* contacts);

/* Snapshot of one world (b2World.Dump b2world.d:796-855 replaced by an exact binary form).
 * Arrays are sized from the header: bodies[body_count], proxies[fixture_count],
 * contacts[contact_count], joints[joint_count].  Pass NULL arrays to read the header only. */
int32_t dbox_world_export_state(dbox_world* w, int32_t world, dbox_world_header* header,
                                dbox_body_state* bodies, dbox_proxy_state* proxies,
                                dbox_contact_state* contacts, dbox_joint_state* joints);
/* Restore a snapshot into a world whose bodies, fixtures and joints were created identically. */
int32_t dbox_world_import_state(dbox_world* w, int32_t world, const dbox_world_header* header,
                                const dbox_body_state* bodies, const dbox_proxy_state* proxies,
                                const dbox_contact_state* contacts, const dbox_joint_state* joints);

/* b2World.GetProfile (b2world.d:789-792): phase times of the last step, summed over worlds. */
int32_t dbox_world_get_profile(dbox_world* w, dbox_profile* out);

/* `steps` steps captured once into one CUDA graph with CUDA events at the phase
 * boundaries of every step; the graph is launched once and waited for.  total_ms
 * receives the device time of all steps, phase_ms[3] the summed time of Collide
 * (+ new-fixture pairs), Solve (islands, solver, broad-phase) and SolveTOI. */
int32_t dbox_world_step_n_timed(dbox_world* w, float dt, int32_t velocity_iterations, int32_t position_iterations,
                                int32_t steps, float* total_ms, float* phase_ms);

/* Cumulative device work counters summed over worlds: out[8] = island bodies integrated,
 * contact constraints built, contact velocity solves, contact position solves, contacts
 * processed by Collide, TOI events, world-steps, broad-phase pairs. */
int32_t dbox_world_get_counters(dbox_world* w, unsigned long long* out);

/* b2Body.ApplyForceToCenter + b2Body.ApplyTorque with wake = false (b2body.d:360-420) for every
 * body of every world: force_torque holds (fx, fy, torque) per body in (world, body id) order. */
int32_t dbox_world_apply_forces(dbox_world* w, const float* force_torque);

/* b2Body.GetPosition + b2Body.GetAngle (b2body.d:283-296) for every body: (x, y, angle) per body. */
int32_t dbox_world_get_transforms(dbox_world* w, float* xya);

/* Per-world device clock figures of the last step (diagnostics): enable before stepping;
 * out receives 32 uint64 per world: slots 0..11 clock stamps at the phase boundaries of the
 * solve kernel, 12..14 the world's velocity levels, contacts and bodies, 16 the cycles of the
 * SolveTOI kernel, 17 its TOI events, 18..24 its cycles per part of the event loop (sweep
 * advance, TOI, minimum, event contact, neighbours, sub-step solve, fixture sync and pairs),
 * 25..26 the global timer (ns) when the world's warp started and ended the solve + SolveTOI
 * kernel, 27 its warp slot, 28..29 the SM and the warp's slot on the SM (%smid, %warpid);
 * 15 for a world solved on a warp 1 when its solver body rows were in shared memory; for a
 * large world (4,096+ fixtures) 15 the cycles of its block's end of Collide, 27 the blocks of
 * its Solve's cluster, 28 the SM of the first, 29 the cycles of SolveTOI's setup passes on its
 * cluster, 30 of its block's SynchronizeFixtures + pair search, 31 of its AddPair pass (25..26
 * unused). */
int32_t dbox_world_set_phase_profile(dbox_world* w, int32_t enable);
int32_t dbox_world_get_phase_profile(dbox_world* w, unsigned long long* out);

/* b2World.Dump (b2world.d:796-855 with b2Body.Dump b2body.d:992-1022, b2Fixture.Dump
 * b2fixture.d:280-358 and the joints' Dump): the text the reference logs, statements that
 * rebuild world `world` with its current positions, angles and velocities (contacts and
 * warm-start impulses are not part of it).  A chain is dumped as its b2ChainShape, a mouse
 * joint as the reference's "not supported" line.  The text is written to buf when capacity
 * > 0 (NUL-terminated, cut at capacity - 1 bytes); out_length receives its full length. */
int32_t dbox_world_dump(dbox_world* w, int32_t world, char* buf, int64_t capacity, int64_t* out_length);

/* The CUDA stream (a cudaStream_t) all device work of the handle is enqueued on, for callers
 * that order their own work or events after it.  No counterpart in the reference. */
int32_t dbox_world_get_stream(dbox_world* w, void** out);

/* Wait for all queued device work of the handle. */
int32_t dbox_world_sync(dbox_world* w);

/* Islands solved and TOI events handled by world `world` in the last step. */
int32_t dbox_world_step_stats(dbox_world* w, int32_t world, int32_t* islands, int32_t* toi_events);

/* ---- World queries, batched (b2World.QueryAABB b2world.d:563-569, b2World.RayCast
 * b2world.d:577-587, over b2DynamicTree.Query / RayCast b2dynamictree.d:203-331).
 * Each query names its world.  The broad-phase's fat AABBs are indexed on the device by a
 * Morton-ordered 32-ary bounding-volume hierarchy, rebuilt on the first query after any
 * step or edit.  The reference reports fixtures in the order of its tree walk and lets the
 * callback stop or clip the walk; here the results are the callback-independent forms:
 *   QueryAABB: every fixture whose fat AABB overlaps the box (b2TestOverlap), in
 *              fixture order (a callback that returns true for each);
 *   RayCast DBOX_RAY_ALL: every fixture the ray hits (b2Fixture.RayCast with maxFraction 1,
 *              the callback returning 1), in fixture order;
 *   RayCast DBOX_RAY_CLOSEST: the hit with the smallest fraction, the lower fixture index on
 *              a tie (the closest-hit callback that returns the fraction).  The tie rule
 *              departs from the reference on purpose: there the clipping callback keeps the
 *              last of several equal-fraction hits in tree-walk order (b2PolygonShape.RayCast
 *              accepts lower == maxFraction), which depends on the tree's shape; this library
 *              keeps the proxy ids and fat AABBs exact but not the tree, so it breaks ties by
 *              fixture index (rays along a shared edge of touching boxes can differ).
 * The testbed's other callbacks (examples/demo/tests/raycast.d) map onto these: the "any hit"
 * callback (returns 0 at its first hit) is DBOX_RAY_ALL with capacity 1, which gives the hit
 * of the lowest fixture index and the number of hits; the "multiple hits" callback (up to N
 * hits, returning 1) is DBOX_RAY_ALL with capacity N, the first N in fixture order.
 * counts[q] receives the number of results of query q (it may exceed capacity; results
 * beyond capacity are dropped; -1: the query names no world, or p1 == p2 for a ray, where
 * the reference asserts); results of query q start at q * capacity, and entries past
 * min(count, capacity) are unspecified. */
#define DBOX_RAY_CLOSEST 0
#define DBOX_RAY_ALL 1
int32_t dbox_world_query_aabb(dbox_world* w, int32_t n, const int32_t* world, const dbox_aabb* boxes,
                              int32_t capacity, int32_t* counts, int32_t* fixtures);
int32_t dbox_world_raycast(dbox_world* w, int32_t n, const int32_t* world, const dbox_vec2* p1, const dbox_vec2* p2,
                           int32_t mode, int32_t capacity, int32_t* counts, dbox_ray_hit* hits);
/* The same with every array in device memory: enqueued on the handle's stream, no wait. */
int32_t dbox_world_query_aabb_device(dbox_world* w, int32_t n, const int32_t* world, const dbox_aabb* boxes,
                                     int32_t capacity, int32_t* counts, int32_t* fixtures);
int32_t dbox_world_raycast_device(dbox_world* w, int32_t n, const int32_t* world, const dbox_vec2* p1,
                                  const dbox_vec2* p2, int32_t mode, int32_t capacity, int32_t* counts,
                                  dbox_ray_hit* hits);

/* Narrowphase alone: the manifolds of n shape pairs at transforms xf = (p.x, p.y, sin, cos), 4 floats
 * per pair, computed on the GPU (b2CollidePolygons collision/b2collidepolygon.d:127-254,
 * b2CollidePolygonAndCircle / b2CollideCircles collision/b2collidecircle.d:29-164).  For a
 * polygon-circle pair the polygon is shape_a.  Only the manifold fields of out are written. */
int32_t dbox_collide_manifolds(int32_t n, const dbox_shape_def* shape_a, const float* xf_a,
                               const dbox_shape_def* shape_b, const float* xf_b, dbox_contact_state* out);

/* Same result as dbox_collide_manifolds, without allocating anything.  No counterpart in
 * the reference (dbox allocates nothing on a GPU).  For callers that must not call
 * cudaMalloc: code in a frame loop with a no-allocation rule, or a process whose device
 * memory belongs to another allocator.  The device memory used lives in one file-scope
 * array of the library (4096 pairs, 1,966,080 bytes), held by every GPU that loads the
 * library until the process exits.  At most 4096 pairs per call (DBOX_ERR_CAPACITY
 * beyond that).  The first call on each device looks up the array's device address,
 * so make that first call before any stream capture.  All calls share the array:
 * calls that overlap on the GPU (several host threads, or several processes sharing a
 * context) race and must be serialised by the caller.  Synchronous on the default stream. */
int32_t dbox_collide_manifolds_noalloc(int32_t n, const dbox_shape_def* shape_a, const float* xf_a,
                                       const dbox_shape_def* shape_b, const float* xf_b, dbox_contact_state* out);

/* ---- Learned warm start (new in this library; dbox has no counterpart) ----
 * A 32 -> 128 -> 128 -> 4 GELU network (BF16 weights and activations, FP32 accumulation, run
 * on the tensor cores) predicts the normal and tangent impulses of manifold points that
 * b2Contact.Update (contacts/b2contact.d:306-324) starts from zero because no feature id
 * matched.  The plain method (mode 0) is the reference step, bit for bit.  Parameters are
 * one flat FP32 vector of DBOX_MLP_PARAMS floats: w1[32][128], w2[128][128], w3[128][8]
 * (columns 4..7 unused), b1[128], b2[128], b3[8]; normalisation is DBOX_MLP_NORM floats:
 * feature mean[32], std[32], target mean[4], std[4].  Samples are DBOX_MLP_SAMPLE floats:
 * 32 features (normal; per point rA, rB, relative normal / tangent velocity, normal mass,
 * tangent mass, velocity bias; inverse masses and inertias; friction, restitution, point
 * count, separations, gravity along the normal times dt, wA, wB) then the 4 impulses the
 * plain solver converged to in that step. */
#define DBOX_MLP_PARAMS 21768
#define DBOX_MLP_NORM 72
#define DBOX_MLP_SAMPLE 36
typedef struct dbox_mlp dbox_mlp;
int32_t dbox_mlp_create(dbox_mlp** out);
int32_t dbox_mlp_destroy(dbox_mlp* m);
int32_t dbox_mlp_init(dbox_mlp* m, uint64_t seed);                       /* uniform fan-in init, zero biases */
int32_t dbox_mlp_set_params(dbox_mlp* m, const float* params, const float* norm);   /* either may be NULL */
int32_t dbox_mlp_get_params(dbox_mlp* m, float* params, float* norm);
int32_t dbox_mlp_fit_normalization(dbox_mlp* m, int32_t n, const float* feats, const float* targets);
/* loss = mean over samples and outputs of (MLP(x) - t)^2 in normalised units; grad = its gradient */
int32_t dbox_mlp_gradient(dbox_mlp* m, int32_t n, const float* feats, const float* targets, float* grad, float* loss);
/* Adam (beta 0.9 / 0.999, eps 1e-8) over shuffled batches; epoch_loss[epochs] (may be NULL) */
int32_t dbox_mlp_train(dbox_mlp* m, int32_t n, const float* feats, const float* targets, int32_t epochs,
                       int32_t batch, float lr, uint64_t seed, float* epoch_loss);
/* The same on n device rows of 36 floats (32 features, 4 targets); device_rows 16-byte aligned. */
int32_t dbox_mlp_train_device(dbox_mlp* m, int32_t n, const float* device_rows, int32_t epochs, int32_t batch,
                              float lr, uint64_t seed, float* epoch_loss);
int32_t dbox_mlp_train_world(dbox_mlp* m, dbox_world* w, int32_t epochs, int32_t batch, float lr, uint64_t seed,
                             float* epoch_loss);                          /* on the world's logged samples */
int32_t dbox_mlp_forward(dbox_mlp* m, int32_t n, const float* feats, float* out);   /* out: n x 4 impulses */
/* mode 0 plain; 1 plain + log up to sample_capacity samples on the device; 2 learned start
 * with `model` (kept by the caller while the mode is on); 3 given start: new points start from
 * the impulses of the same contact slot in the handle named by dbox_world_set_start_source
 * (for measuring what a perfect prediction would give: that handle steps the same state with
 * more iterations first).  In mode 2 the first velocity iteration keeps, per contact, the
 * start (predicted or zero) whose first correction is smaller.  Modes 1 to 3 set contact flags
 * 0x40 / 0x80 (point 0 / 1 new this step). */
int32_t dbox_world_set_warmstart(dbox_world* w, int32_t mode, dbox_mlp* model, int32_t sample_capacity);
/* Mode 3's source: a handle of the same worlds, laid out the same way (created from the same
 * scenes and sizing hints, no edits since); read during each step of w.  No counterpart in
 * the reference. */
int32_t dbox_world_set_start_source(dbox_world* w, dbox_world* src);
/* Exact copy of the simulation state of src into dst, device to device (bodies, proxies,
 * contacts with their warm-start impulses, joints, the pair table): the checkpoint of
 * dbox_world_export_state / import_state without a host round trip, for handles of the same
 * worlds laid out the same way.  No counterpart in the reference. */
int32_t dbox_world_copy_state(dbox_world* dst, dbox_world* src);
int32_t dbox_world_sample_count(dbox_world* w, int32_t* count);
int32_t dbox_world_get_samples(dbox_world* w, int32_t offset, int32_t n, float* rows);  /* n x 36 */
int32_t dbox_world_clear_samples(dbox_world* w);
/* Solver quality of each step while enabled: out[4 per world] = sum over contact points of
 * |lambda_next - lambda|^2 from one extra non-mutating velocity sweep after the last
 * iteration, its maximum, the number of points, and the minimum separation after the step. */
int32_t dbox_world_set_measure(dbox_world* w, int32_t enable);
int32_t dbox_world_get_quality(dbox_world* w, float* out);

/* Mapping of the worlds onto the solve kernel (new; no counterpart in dbox): warp slots
 * (worlds) per block, 1, 2 or 4, and the per-block budget of solver body rows in shared
 * memory, in bodies (0 = chosen from the worlds).  Results do not depend on it. */
int32_t dbox_world_set_mapping(dbox_world* w, int32_t warps_per_block, int32_t body_budget);
/* The same, with the `isolate` largest worlds each given a block of its own. */
int32_t dbox_world_set_mapping_isolated(dbox_world* w, int32_t warps_per_block, int32_t body_budget, int32_t isolate);
/* World-queue mapping: one resident wave of warps takes worlds from a queue, costliest first
 * (the costs given by dbox_world_set_world_costs, else body counts); the `heavy` costliest
 * worlds go one per SM sub-partition at a time, and with `exclusive` a warp whose
 * sub-partition runs a heavy world waits (bounded) before it takes another world;
 * blocks_per_sm limits the resident four-warp blocks per SM (0: as many as fit).  Worlds
 * of up to about 580 bodies keep their solver rows in shared memory.  Results do not depend
 * on the mapping. */
int32_t dbox_world_set_mapping_queue(dbox_world* w, int32_t heavy, int32_t exclusive, int32_t blocks_per_sm);
/* Per-world cost estimates (n_worlds floats; NULL clears them) for the queue order. */
int32_t dbox_world_set_world_costs(dbox_world* w, const float* cost);
/* The per-world costs in use (measured by the autotuner, or given; else body counts). */
int32_t dbox_world_get_world_costs(dbox_world* w, float* out);
/* Autotuner: measures each world's warp time in one profiled step (kept as the queue
 * costs), then times `steps` steps (the simulation advances) under each candidate mapping,
 * twice, and keeps the fastest; choice[6] receives (warps per block, body budget, isolated,
 * queue, heavy, exclusive): the first three for a block packing (queue = 0), the last two
 * for a queue mapping (queue = 1).  With large worlds (4,096+ fixtures) it then times their
 * Solve on a block and on a warp the same way and keeps the faster island solver
 * (dbox_world_get_island_solver). */
int32_t dbox_world_autotune(dbox_world* w, float dt, int32_t velocity_iterations, int32_t position_iterations,
                            int32_t steps, int32_t* choice);

/* Budget of one bounded device wait (no counterpart in the reference): the solve kernel waits
 * on an mbarrier for each block of constraint rows it copies into shared memory; a wait that
 * takes more than `polls` polls (default and maximum 2^20) makes the step return
 * DBOX_ERR_TIMEOUT.  The wait itself goes on until the copy has landed (up to 2^20 polls), so the
 * step's results are unaffected; a lower budget lets a caller check its handling of the error. */
int32_t dbox_world_set_wait_limit(dbox_world* w, int32_t polls);

/* How b2World.Solve runs for the large worlds of the handle (4,096 fixtures or more): mode 0
 * (default) on a thread-block cluster of up to 8 blocks of 1,024 threads each (islands found by
 * a union-find, each island's search on a thread of its own, the parallel phases and the
 * constraint level sweeps spread over the cluster), mode 1 on one warp each like every other
 * world.  Both give the same results bit for bit, in every warm-start mode
 * (dbox_world_set_warmstart 0..3).  Replaces no reference call: the
 * reference solves islands one after another on the calling thread (dynamics/b2world.d:930-1124). */
int32_t dbox_world_set_island_solver(dbox_world* w, int32_t mode);
/* The mode in use (set by the call above or chosen by dbox_world_autotune). */
int32_t dbox_world_get_island_solver(dbox_world* w, int32_t* mode);

/* Whole steps in one launch (no counterpart in the reference, which steps one world on the
 * calling thread: dynamics/b2world.d:367-434): with enable = 1 (default 0) a handle without large
 * worlds (4,096+ fixtures) and without a PreSolve window runs each step as one kernel in which
 * every world's warp goes from its Collide straight to its Solve and SolveTOI, and
 * dbox_world_step_n / dbox_world_step_n_timed run all their steps in one such launch (each world
 * takes its steps one after the other; separate worlds share nothing, so no world waits at a
 * step boundary for the others).  The results are the same bits as the per-phase launches
 * (enable = 0: 4 launches a step).  With the fused launch dbox_world_step_n_timed reports the
 * whole step as its phase 1 and dbox_world_get_profile only the step time. */
int32_t dbox_world_set_fused_step(dbox_world* w, int32_t enable);
int32_t dbox_world_get_fused_step(dbox_world* w, int32_t* enable);

/* Device kernels launched by the last stepping call (dbox_world_step, dbox_world_step_n or
 * dbox_world_step_n_timed, all of its steps; for launch accounting). */
int32_t dbox_world_last_launches(dbox_world* w, int32_t* out);

/* Text of the last error on the calling thread (never NULL). */
const char* dbox_last_error(void);

#ifdef __cplusplus
}
#endif

#endif /* DBOX_GPU_H */
