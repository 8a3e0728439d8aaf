/*
 * pk_oracle.h — C interface of the FP64 CPU oracle for the PhysKit world step.
 *
 * TEST INFRASTRUCTURE ONLY. The oracle is a dependency-free C++20 restatement of the
 * reference's world-step path (src/world.cpp:20-56 and everything it calls). It is the
 * checker for the CUDA implementation in physkit_gb300/ and the timed CPU baseline in
 * bench.py. Nothing in the product links, loads or calls it.
 *
 * Parity is pinned against the reference's own known-answer tests
 * (tests/gjk/gjk_test.cpp, tests/epa/epa_test.cpp, tests/dynamic_bvh/main.cpp,
 * tests/mesh/main.cpp, tests/obb/obb_test.cpp), restated under tests/.
 * The reference itself cannot be compiled here (C++26, Eigen 5, mp-units, abseil).
 */
#ifndef PK_ORACLE_H
#define PK_ORACLE_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct pko_world pko_world;

/* Solver contact order. KEY: manifolds in ascending pair-key order, contacts in manifold order
 * (the reference's sequential Gauss-Seidel with its hash-set order made deterministic).
 * COLOUR: manifolds grouped by the deterministic min-index claiming colouring that the GPU
 * solver uses, colours ascending, manifolds ascending inside a colour. */
enum { PKO_ORDER_KEY = 0, PKO_ORDER_COLOUR = 1 };

pko_world *pko_world_create(double gx, double gy, double gz, int solver_iterations, int order);
void pko_world_destroy(pko_world *w);

/* Shapes (meshes, shared by bodies). Returns shape id >= 0 or -1. */
int pko_shape_box(pko_world *w, double hx, double hy, double hz);
int pko_shape_sphere(pko_world *w, double radius, int stacks, int sectors);
int pko_shape_pyramid(pko_world *w, double base_half, double height);
int pko_shape_mesh(pko_world *w, const double *verts, int nverts, const int *tris, int ntris);
int pko_shape_vertex_count(pko_world *w, int shape);
int pko_shape_triangles(pko_world *w, int shape, int *out, int cap); /* 3 vertex indices each; returns the count */
int pko_shape_vertices(pko_world *w, int shape, double *out, int cap);
double pko_shape_volume(pko_world *w, int shape);

/* Body creation mirrors world_base::create_rigid (world.h:202-208).
 * quat is (w,x,y,z); inertia is row-major 3x3. Returns the arena handle id
 * (idx | gen<<32) or UINT64_MAX on invalid input. */
uint64_t pko_body_add(pko_world *w, int is_static, const double *pos, const double *quat,
                      const double *vel, const double *ang_vel, double mass,
                      const double *inertia, double restitution, double friction, int shape);
int pko_body_remove(pko_world *w, uint64_t handle);
int pko_body_count(pko_world *w); /* number of arena slots (alive or free) */

void pko_world_step(pko_world *w, double dt);

/* Per slot: pos3 quat4(wxyz) vel3 angvel3 alive(1) = 14 doubles. Returns slot count. */
int pko_read_bodies(pko_world *w, double *out, int cap_slots);
/* Overwrite the dynamic state of one slot (pos3, quat4, vel3, angvel3) and refresh cached
 * inertia; used to start GPU and oracle from the same snapshot. */
int pko_write_body_state(pko_world *w, int slot, const double *state13);
/* Sorted active broadphase pair keys ((min<<32)|max). Returns count (may exceed cap). */
int pko_read_pairs(pko_world *w, uint64_t *keys, int cap);
/* Manifolds in key order. Per manifold: key(as double bits in a uint64 array) is written to
 * keys; per contact 13 doubles: normal3 local_a3 local_b3 depth normal_imp t1_imp t2_imp.
 * counts[i] = number of contacts. contacts has room for 4 per manifold. */
int pko_read_manifolds(pko_world *w, uint64_t *keys, int *counts, double *contacts, int cap);
/* Events of the last step in narrowphase order: key and kind (1 begin, 2 end). */
int pko_read_events(pko_world *w, uint64_t *keys, int *kinds, int cap);
/* Joints (constraint.h:139-865), type 0 distance 1 ball_socket 2 hinge 3 slider 4 weld 5 spring.
 * p18: anchor3 local_a3 local_b3 axis_a3 axis_b3 distance stiffness damping. Returns the handle
 * (slot | gen << 32 | type << 56). pko_joint_impulses: the accumulated impulses, returns the row count. */
uint64_t pko_joint_add(pko_world *w, int type, uint64_t a, uint64_t b, const double *p18);
int pko_joint_remove(pko_world *w, uint64_t handle);
int pko_joint_impulses(pko_world *w, uint64_t handle, double *out6);
/* world_base::raycast (world.h:260-319): hits in the reference's order; returns the hit count */
/* mesh::instance::ray_intersect (mesh.cpp:400-415) of shape at pose7 (pos3, quat wxyz): 1 with
 * out7 = hit pos3, normal3, distance and the triangle index; 0 on a miss. */
int pko_mesh_raycast(pko_world *w, int shape, const double *pose7, const double *origin, const double *dir,
                     double max_dist, double *out7, int *tri);
int pko_world_raycast(pko_world *w, const double *origin, const double *dir, double max_dist, uint64_t *handles,
                      double *dist, int cap);
/* Colour of each active manifold of the last step (key order) and the colour count. */
int pko_read_colours(pko_world *w, uint64_t *keys, int *colours, int cap, int *ncolours);
/* Number of reinsertions (moved leaves) of the last step. */
int pko_last_moved(pko_world *w);

/* Narrowphase on primitive shapes, for the reference's GJK/EPA known answers.
 * kind: 0 aabb (params min3 max3), 1 obb (center3 quat4 half3), 2 mesh instance
 * (pos3 quat4, shape id in the world given). out: normal3 world_a3 world_b3 depth.
 * Returns 1 on collision, 0 otherwise. */
int pko_gjk_epa(pko_world *w, int kind_a, const double *pa, int shape_a, int kind_b,
                const double *pb, int shape_b, double *out);

/* Standalone dynamic AABB tree (dynamic_bvh, bvh.h:270-535) for the tree known answers. */
typedef struct pko_tree pko_tree;
pko_tree *pko_tree_create(void);
void pko_tree_destroy(pko_tree *t);
uint32_t pko_tree_add(pko_tree *t, uint32_t id, const double *box6);
int pko_tree_update(pko_tree *t, uint32_t leaf, const double *box6, const double *disp3);
void pko_tree_remove(pko_tree *t, uint32_t leaf);
void pko_tree_bounds(pko_tree *t, uint32_t leaf, double *box6);
int pko_tree_query(pko_tree *t, const double *box6, uint32_t *out, int cap);
int pko_tree_height(pko_tree *t);
int pko_tree_validate(pko_tree *t); /* 1 when parent links, heights and bounds are consistent */

/* Deterministic half-angle sine/cosine used by the orientation update (exposed for tests). */
void pko_sincos(double x, double *s, double *c);

#ifdef __cplusplus
}
#endif
#endif
