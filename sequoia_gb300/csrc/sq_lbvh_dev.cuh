// sq_lbvh_dev.cuh -- device helpers of the LBVH climb shared by the
// single-mesh (sq_lbvh.cu) and batched (sq_batch.cu) builders.
#pragma once

#include "sq_common.cuh"

namespace sq {

// Mesh of position i in a batch whose mesh m holds positions
// [off[m], off[m + 1]): the largest m < M with off[m] <= i.
__device__ __forceinline__ uint32_t mesh_of(const uint32_t* __restrict__ off, uint32_t M, uint32_t i)
{
    uint32_t lo = 0, hi = M;
    while (hi - lo > 1) {
        const uint32_t mid = (lo + hi) >> 1;
        if (__ldg(off + mid) <= i) lo = mid; else hi = mid;
    }
    return lo;
}

struct RunFrame {
    uint32_t b, e, slot, state;
    Box acc;
};

// Halving subtree of a run of >= 8 equal codes over [b0, e0)
// (find_split_morton's equal-codes case, src/builder.cpp:2288-2289).  Writes
// every record strictly inside the run; returns the run's box and split.
__device__ inline void run_subtree(uint32_t b0, uint32_t e0, uint32_t leaf0, Node* __restrict__ nodes, Box& out_box,
                            uint32_t& out_split, uint32_t* err)
{
    RunFrame st[40];
    int sp = 0;
    st[0].b = b0; st[0].e = e0; st[0].slot = 0xFFFFFFFFu; st[0].state = 0;
    box_reset(st[0].acc);
    sp = 1;
    while (sp > 0) {
        RunFrame& f = st[sp - 1];
        const uint32_t c = f.e - f.b;
        if (c < 8) {
            Box bb;
            box_reset(bb);
            for (uint32_t p = f.b; p < f.e; ++p) {
                const float4 a = reinterpret_cast<const float4*>(nodes + leaf0 + p)[0];
                const float4 z = reinterpret_cast<const float4*>(nodes + leaf0 + p)[1];
                Box lb;
                lb.mn[0] = a.x; lb.mn[1] = a.y; lb.mn[2] = a.z;
                lb.mx[0] = z.x; lb.mx[1] = z.y; lb.mx[2] = z.z;
                box_grow(bb, lb);
            }
            store_node(nodes + f.slot, bb, leaf0 + f.b, c, 0);
            --sp;
            box_grow(st[sp - 1].acc, bb);
            continue;
        }
        const uint32_t q = f.b + (c >> 1) + 1u;
        if (f.state == 0) {
            f.state = 1;
            if (sp >= 40) { raise_error(err, SQ_DEVERR_TOPOLOGY); return; }
            RunFrame& g = st[sp++];
            g.b = f.b; g.e = q; g.slot = 2u * q; g.state = 0;
            box_reset(g.acc);
        } else if (f.state == 1) {
            f.state = 2;
            if (sp >= 40) { raise_error(err, SQ_DEVERR_TOPOLOGY); return; }
            RunFrame& g = st[sp++];
            g.b = q; g.e = f.e; g.slot = 2u * q + 1u; g.state = 0;
            box_reset(g.acc);
        } else {
            if (f.slot == 0xFFFFFFFFu) {
                out_box = f.acc;
                out_split = q;
                return;
            }
            store_node(nodes + f.slot, f.acc, 2u * q, 2u, 0);
            const Box done = f.acc;
            --sp;
            box_grow(st[sp - 1].acc, done);
        }
    }
}

// Record of a child over [cl, cr) (count cc) in the parent's slot.
__device__ __forceinline__ void write_child(Node* __restrict__ nodes, uint32_t slot, uint32_t cl, uint32_t cr,
                                            const Box& b, uint32_t split, uint32_t leaf0)
{
    const uint32_t cc = cr - cl;
    if (cc >= 8) {
        store_node(nodes + slot, b, 2u * split, 2u, 0);
    } else if (cc >= 2) {
        store_node(nodes + slot, b, leaf0 + cl, cc, 0);
    } else {
        const float4* src = reinterpret_cast<const float4*>(nodes + leaf0 + cl);
        const float4 a = __ldcg(src), z = __ldcg(src + 1);
        reinterpret_cast<float4*>(nodes + slot)[0] = a;
        reinterpret_cast<float4*>(nodes + slot)[1] = z;
    }
}

}  // namespace sq
