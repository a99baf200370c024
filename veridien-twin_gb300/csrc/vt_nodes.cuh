// Launchers of the node radiosity kernels (vt_nodes.cu).
#pragma once

#include "vt_device.cuh"

namespace vtk {

// gather table of n_nodes x K rays (build, escape count into aux[i].x, remap to active nodes)
void launch_gather_build(const vtd::Scene& S, uint32_t n_nodes, uint32_t K, uint32_t* gtable, float4* aux, cudaStream_t st);
// A(mu_in) of each gather ray per material: n_mat x K
void launch_amu(const vtd::Scene& S, uint32_t n_mat, uint32_t K, float4* amu, cudaStream_t st);
// the node direct light (nodeDirect) in three passes; work: node_direct_bytes(n_active, NS) of device memory
struct NodeDirectBufs {
  float4* ro;         // per (node, sample): shadow ray origin | its length
  float4* rd;         // direction
  float4* term;       // the sample's unshadowed term | flags (lit, visible, node updated)
  uint32_t* queue;    // the lit samples
  uint32_t* counts;   // queued, taken
};
size_t node_direct_bytes(uint32_t n_active, uint32_t NS);
// trace_blocks: the persistent shadow lanes' grid (blocks of 256)
void launch_node_direct(const vtd::Scene& S, const uint32_t* active, uint32_t n_active, uint32_t NS, uint32_t moved, float4* nstate, void* work,
                        int trace_blocks, cudaStream_t st);
// transport table: landing rays per active node, then the rows (row: n_active + 1 offsets, exclusive)
void launch_transport_count(const uint32_t* active, uint32_t n_active, uint32_t K, const uint32_t* gtable, uint32_t* cnt, cudaStream_t st);
void launch_transport_fill(const vtd::Scene& S, const uint32_t* active, uint32_t n_active, uint32_t K, const uint32_t* gtable, const float4* amu,
                           const uint32_t* row, float4* ent, cudaStream_t st);
// one Jacobi step: gather from slot_in into aux (from the transport table when ent is set, else evaluating each
// ray's factor), update into slot_out
void launch_jacobi_step(const vtd::Scene& S, const uint32_t* active, uint32_t n_active, uint32_t K, const uint32_t* gtable, const float4* amu,
                        const uint32_t* row, const float4* ent, const uint2* nbr, uint32_t nbr_k, uint32_t slot_in, uint32_t slot_out,
                        float4* nstate, float4* aux, cudaStream_t st);

}  // namespace vtk
