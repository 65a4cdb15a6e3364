/*
 * b2_oracle.h - TEST INFRASTRUCTURE ONLY.
 *
 * CPU restatement of dbox's b2World.Step (dbox is a D port of Box2D 2.3.1),
 * used as the parity checker for the GPU library and as the timed CPU
 * baseline.  Only tests/, __graft_entry__.smoke() and bench.py's CPU legs may
 * load it.  The product (libdbox_gpu.so) never links or calls it.
 *
 * Parity status: the reference ships no tests, fixtures or recorded outputs and
 * no D compiler exists on either machine, so this restatement is checked
 * against its own known-answer cases (tests/golden) and invariants; parity is
 * "unpinned" in the sense that no output of the reference itself was compared.
 *
 * Trig: the reference calls the C runtime's sinf/cosf (common/b2math.d:478-488).
 * orc_set_trig_mode(0) uses the host libm (reference semantics, the default);
 * orc_set_trig_mode(1) uses dbox_sincosf from dbox_gb300/csrc/dbox_trig.h,
 * which the GPU library also uses, so trajectories can be compared bit for bit.
 */
#ifndef B2_ORACLE_H
#define B2_ORACLE_H

#include "../include/dbox_gpu.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct orc_world orc_world;

void orc_set_trig_mode(int mode);
int orc_get_trig_mode(void);

orc_world* orc_world_create(float gx, float gy);
void orc_world_destroy(orc_world* w);
int orc_body_create(orc_world* w, const dbox_body_def* def);
int orc_fixture_create(orc_world* w, int body, const dbox_shape_def* shape, const dbox_fixture_def* def);
int orc_joint_create_revolute(orc_world* w, const dbox_revolute_def* def);
int orc_world_dump(orc_world* w, char* buf, int cap);
int orc_joint_create_gear(orc_world* w, const dbox_gear_def* def);
int orc_body_destroy(orc_world* w, int body);
int orc_fixture_destroy(orc_world* w, int fixture);
int orc_joint_destroy(orc_world* w, int joint);
int orc_query_aabb(orc_world* w, float lx, float ly, float ux, float uy, int* out, int cap);
void orc_raycast_many(orc_world* w, int n, const float* p1, const float* p2, int mode, int* counts, dbox_ray_hit* hits,
                      int cap);
void orc_query_aabb_many(orc_world* w, int n, const float* boxes, int* counts, int* out, int cap);
int orc_raycast(orc_world* w, float x1, float y1, float x2, float y2, int mode, dbox_ray_hit* out, int cap);
int orc_fixture_create_chain(orc_world* w, int body, const dbox_vec2* vertices, int count, int loop,
                             const dbox_vec2* prev, const dbox_vec2* next, const dbox_fixture_def* def);
int orc_joint_create_distance(orc_world* w, const dbox_distance_def* def);
int orc_joint_create_rope(orc_world* w, const dbox_rope_def* def);
int orc_joint_create_weld(orc_world* w, const dbox_weld_def* def);
int orc_joint_create_friction(orc_world* w, const dbox_friction_def* def);
int orc_joint_create_motor(orc_world* w, const dbox_motor_def* def);
int orc_joint_create_wheel(orc_world* w, const dbox_wheel_def* def);
int orc_joint_create_prismatic(orc_world* w, const dbox_prismatic_def* def);
int orc_joint_create_pulley(orc_world* w, const dbox_pulley_def* def);
int orc_joint_create_mouse(orc_world* w, const dbox_mouse_def* def);
int orc_joint_set_mouse_target(orc_world* w, int joint, float x, float y);
int orc_scene_create(orc_world* w, int n_bodies, const dbox_body_def* bodies, int n_fixtures,
                     const int* fixture_body, const dbox_shape_def* shapes, const dbox_fixture_def* fixtures,
                     int n_joints, const dbox_revolute_def* joints);
void orc_world_set_flags(orc_world* w, int warm, int continuous, int substep, int sleep, int autoclear);
void orc_world_step(orc_world* w, float dt, int vel_iters, int pos_iters);
void orc_world_step_n(orc_world* w, float dt, int vel_iters, int pos_iters, int steps);

/* record contact events (Begin/End/PreSolve/PostSolve) into an internal log */
void orc_world_record_events(orc_world* w, int enable);
int orc_world_event_count(orc_world* w);
int orc_world_get_events(orc_world* w, dbox_contact_event* out, int cap);
void orc_world_clear_events(orc_world* w);
/* a user PreSolve (b2ContactListener.PreSolve) called with one record per call, inside Collide
 * and SolveTOI as the reference calls it; its edits are applied to the contact.  The record's
 * world is 0 for a call from Collide and -1 for one from SolveTOI's sub-step updates. */
void orc_world_set_presolve(orc_world* w, dbox_presolve_fn fn, void* user);
/* b2Fixture.SetFilterData + Refilter; a user b2ContactFilter over a class table (the
 * fixture's class stands in for the user data such a filter reads), optionally with the
 * default rule; table NULL restores b2_defaultFilter */
int orc_fixture_set_filter(orc_world* w, int fixture, int category, int mask, int group);
int orc_fixture_set_filter_class(orc_world* w, int fixture, int cls);
void orc_world_set_contact_filter(orc_world* w, const uint64_t* table, int with_default);

int orc_world_export_state(orc_world* w, dbox_world_header* header, dbox_body_state* bodies,
                           dbox_proxy_state* proxies, dbox_contact_state* contacts, dbox_joint_state* joints);

/* last-step diagnostics: number of TOI events, islands */
int orc_world_last_toi_events(orc_world* w);
int orc_world_last_islands(orc_world* w);

/* polygon helper: b2PolygonShape.Set; writes count, vertices, normals, centroid; returns count */
int orc_polygon_set(const float* xy, int n, float* out_vertices, float* out_normals, float* out_centroid);

/* narrowphase entry for known-answer tests: kind 0 circles, 1 polygon-circle, 2 polygons */
int orc_collide(const dbox_shape_def* a, const float* xfa, const dbox_shape_def* b, const float* xfb,
                dbox_contact_state* out_manifold);

/* sin/cos through the selected trig mode */
void orc_sincos(float a, float* s, float* c);
void orc_sincos_array(int n, const float* a, float* s, float* c);

#ifdef __cplusplus
}
#endif
#endif
