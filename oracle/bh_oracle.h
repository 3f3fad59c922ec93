/*
 * bh_oracle.h — CPU oracle of the gkane1234/gravity Barnes–Hut step.
 *
 * TEST INFRASTRUCTURE ONLY.  This is a plain-C restatement of the reference's
 * GLSL compute pipeline, used by tests/ as the checker of the CUDA path, by
 * __graft_entry__.smoke() and by bench.py's CPU-baseline leg.  The product
 * (gravity_gb300, libgbh.so) never links, loads or calls it.
 *
 * Parity status: the reference ships no tests, golden vectors or fixtures and
 * cannot run on these machines (Java + OpenGL).  This restatement is pinned
 * (a) by known-answer tests from the mathematics and (b), in the development
 * container only, against the reference's own GLSL kernel sources compiled as
 * C++ under a hand-written shim (oracle/ref_harness), whose outputs are
 * committed as golden vectors under tests/golden/.
 *
 * Arithmetic: IEEE-754 FP32 with no FMA contraction (-ffp-contract=off) and
 * IEEE division; GLSL inversesqrt is restated as 1.0f/sqrtf(x).
 *
 * The API mirrors include/gbh.h (same structs, same stage boundaries as the
 * reference's BarnesHut.step, BarnesHut.java:99-164).
 */
#ifndef BH_ORACLE_H
#define BH_ORACLE_H

#include <stdint.h>
#include "../include/gbh.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct orc_ctx orc_ctx;

orc_ctx* orc_create(uint32_t initial_num_bodies, const float bounds[6], const gbh_units* units);
void orc_destroy(orc_ctx* c);
void orc_set_threads(int threads);
int orc_get_threads(void);

int orc_upload_bodies(orc_ctx* c, const gbh_body* host, uint32_t count, uint32_t offset);
int orc_init(orc_ctx* c);
int orc_step(orc_ctx* c, const gbh_step_params* p);

/* reference stage boundaries (BarnesHut.java:99-164) */
int orc_stage_reset(orc_ctx* c, const gbh_step_params* p);     /* bh_update.comp reset */
int orc_stage_partition(orc_ctx* c);                            /* bh_dead.comp + swap */
int orc_stage_decrement(orc_ctx* c);                            /* bh_update.comp decrement */
int orc_stage_bounds(orc_ctx* c);                               /* bh_morton.comp:114-231 */
int orc_stage_encode(orc_ctx* c);                               /* bh_morton.comp:238-262 */
int orc_stage_sort(orc_ctx* c);                                 /* bh_radix.comp */
int orc_stage_build(orc_ctx* c);                                /* bh_tree.comp:43-133 */
int orc_stage_fill(orc_ctx* c);                                 /* bh_tree.comp:140-259 */
int orc_stage_walk(orc_ctx* c, const gbh_step_params* p);       /* bh_force.comp:40-142 */
int orc_stage_merge(orc_ctx* c);                                /* bh_merge.comp:30-71 */
int orc_stage_swap(orc_ctx* c);                                 /* GPU.swapBodyBuffers */
/* the walk over every `stride`-th live sorted slot only (CPU-baseline samples);
 * writes nothing to the body buffers */
int orc_stage_walk_sample(orc_ctx* c, const gbh_step_params* p, uint32_t stride, uint64_t* interactions);
/* the sharded step (gbh_step_shard_* of the C ABI, restated) */
int orc_step_shard_walk(orc_ctx* c, const gbh_step_params* p, uint32_t rank, uint32_t world, uint32_t range[2]);
int orc_shard_pack(orc_ctx* c, uint32_t lo, uint32_t count, gbh_body* out);
int orc_shard_unpack(orc_ctx* c, uint32_t lo, uint32_t count, const gbh_body* body);
int orc_read_merge_tasks_full(orc_ctx* c, uint32_t* pairs, uint64_t* keys, uint32_t capacity, uint32_t* count);
int orc_write_merge_tasks(orc_ctx* c, const uint32_t* pairs, const uint64_t* keys, uint32_t count);
int orc_step_shard_finish(orc_ctx* c, uint32_t oob_other_ranks);

int orc_read_bodies(orc_ctx* c, uint32_t which, gbh_body* host, uint32_t count, uint32_t offset);
int orc_read_leaf_nodes(orc_ctx* c, gbh_node* host, uint32_t count, uint32_t offset);
int orc_read_internal_nodes(orc_ctx* c, gbh_node* host, uint32_t count, uint32_t offset);
int orc_read_sim_values(orc_ctx* c, gbh_sim_values* host);
int orc_read_index(orc_ctx* c, uint32_t* host, uint32_t count, uint32_t offset);
int orc_read_morton(orc_ctx* c, uint64_t* host, uint32_t count, uint32_t offset);
int orc_read_merge_tasks(orc_ctx* c, uint32_t* host_pairs, uint32_t capacity, uint32_t* count);
int orc_read_accel(orc_ctx* c, float* host_xyzw, uint32_t count, uint32_t offset);
int orc_read_stats(orc_ctx* c, gbh_stats* host);
int orc_write_sim_values(orc_ctx* c, const gbh_sim_values* host);
int orc_write_index(orc_ctx* c, const uint32_t* host, uint32_t count, uint32_t offset);
int orc_write_morton(orc_ctx* c, const uint64_t* host, uint32_t count, uint32_t offset);

/* FP64 direct sum for `count` sampled body indices over all non-empty bodies
 * of `bodies[0..n)` (self excluded).  out: double[3*count]. */
int orc_direct_sum_fp64(const gbh_body* bodies, uint32_t n, const uint32_t* sample, uint32_t count,
                        double G, double softening, double* out);

/* building blocks, exported for known-answer tests */
uint64_t orc_expand_bits21(uint32_t v);
uint64_t orc_morton3d64(uint32_t x, uint32_t y, uint32_t z);
uint64_t orc_morton_encode(const float pos[3], const float bmin[3], const float bmax[3]);
int orc_safe_lcp(const uint64_t* keys, int n, int i, int j);
void orc_star_color(float mass, float density, float rgb[3]);

/* Level-of-detail node selection of the render shaders, restated: the
 * hierarchical node glow (nodeglow.vert:46-150) and the region boxes
 * (regions.vert:19-45) over internal[0..count), the live internal nodes.
 * `bodies` is the state's body buffer (for view->relative_to) and
 * `num_bodies_cap` its length (initial_num_bodies).  Records are written in
 * node order, at most `capacity`; the return value is the number selected. */
uint32_t orc_select_glow_nodes(const gbh_node* internal, uint32_t count, const gbh_body* bodies,
                               uint32_t num_bodies_cap, const gbh_view* view, gbh_glow_splat* out,
                               uint32_t capacity);
uint32_t orc_select_regions(const gbh_node* internal, uint32_t count, const gbh_body* bodies,
                            uint32_t num_bodies_cap, const gbh_view* view, gbh_region* out, uint32_t capacity);

#ifdef __cplusplus
}
#endif

#endif
