// k_shard.cu — the device half of the sharded step (gbh_step_shard_walk,
// gbh_shard_pack / gbh_shard_unpack, gbh_step_shard_finish).
//
// Every rank builds the same tree (the stages before the walk are
// deterministic), walks its share of the live bodies (shard_slots in
// gbh_common.cuh), and then receives the other ranks' updated bodies.  The
// reference walks every body independently of the others
// (SH/compute/force/bh_force.comp:40-142), so a walk split by body equals the
// whole walk body for body.  The updated bodies travel in sorted-slot order:
// packed[i] = the output body of slot lo + i (32 bytes), followed by the
// count magnitudes |a| of their walk (4 bytes each), which the learned
// criterion reads in the next step (feature 8).
#include "gbh_common.cuh"

// The slots the walk updated: the plain walk its share [lo, hi); the group
// walks every group whose first slot lies in the share, which covers the
// slots from the first group start at or after lo to the first at or after hi.
__global__ void k_shard_range_init(StepBuffers b) {
    const uint32_t n = b.st->n_new;
    uint32_t lo, hi;
    shard_slots(b, n, lo, hi);
    b.st->shard_lo = lo;
    b.st->shard_hi = hi;
}

__global__ void k_shard_range_groups(StepBuffers b) {
    const uint32_t n = b.st->n_new;
    uint32_t lo, hi;
    shard_slots(b, n, lo, hi);
    const uint32_t ng = b.st->num_groups;
    for (uint32_t t = blockIdx.x * blockDim.x + threadIdx.x; t < ng; t += gridDim.x * blockDim.x) {
        const uint32_t first = b.groups[t].x;
        if (first >= lo) atomicMin(&b.st->shard_lo, first);
        if (first >= hi) atomicMin(&b.st->shard_hi, first);
    }
}

__global__ void k_shard_range_groups_init(StepBuffers b) {
    const uint32_t n = b.st->n_new;
    b.st->shard_lo = n;
    b.st->shard_hi = n;
}

void launch_shard_range(const StepBuffers& b, bool groups, cudaStream_t s) {
    if (!groups) {
        k_shard_range_init<<<1, 1, 0, s>>>(b);
        return;
    }
    k_shard_range_groups_init<<<1, 1, 0, s>>>(b);
    k_shard_range_groups<<<b.num_sms * 4, 256, 0, s>>>(b);
}

__global__ void k_shard_pack(StepBuffers b, uint32_t lo, uint32_t count, gbh_body* __restrict__ out) {
    float* mag = reinterpret_cast<float*>(out + count);
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < count; i += gridDim.x * blockDim.x) {
        const uint32_t bi = b.idx_in[lo + i];
        st_body(out, i, ld_pos_mass(b.bodies_out, bi), ld_vel_density(b.bodies_out, bi));
        mag[i] = b.accel_mag[bi];
    }
}

// the other ranks' bodies into the output buffer, and their positions into
// the in-order copy the next compaction reads
__global__ void k_shard_unpack(StepBuffers b, uint32_t lo, uint32_t count, const gbh_body* __restrict__ in) {
    const float* mag = reinterpret_cast<const float*>(in + count);
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < count; i += gridDim.x * blockDim.x) {
        const uint32_t bi = b.idx_in[lo + i];
        const float4 pm = ld_pos_mass(in, i);
        st_body(b.bodies_out, bi, pm, ld_vel_density(in, i));
        b.sorted_pm[lo + i] = pm;
        b.accel_mag[bi] = mag[i];
    }
}

__global__ void k_shard_add_oob(StepBuffers b, uint32_t oob) {
    b.sim->out_of_bounds += oob;
    b.st->oob += oob;
}

static uint32_t copy_blocks(const StepBuffers& b, uint32_t count) {
    const uint32_t need = (count + 255) / 256;
    const uint32_t cap = b.num_sms * 8;
    return need < 1 ? 1 : (need < cap ? need : cap);
}

void launch_shard_pack(const StepBuffers& b, uint32_t lo, uint32_t count, gbh_body* out, cudaStream_t s) {
    if (count) k_shard_pack<<<copy_blocks(b, count), 256, 0, s>>>(b, lo, count, out);
}

void launch_shard_unpack(const StepBuffers& b, uint32_t lo, uint32_t count, const gbh_body* in, cudaStream_t s) {
    if (count) k_shard_unpack<<<copy_blocks(b, count), 256, 0, s>>>(b, lo, count, in);
}

void launch_shard_add_oob(const StepBuffers& b, uint32_t oob, cudaStream_t s) {
    if (oob) k_shard_add_oob<<<1, 1, 0, s>>>(b, oob);
}
