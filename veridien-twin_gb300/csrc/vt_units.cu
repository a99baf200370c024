// The reference's GPU unit kernels (gpu/wgsl/kernels.wgsl.js:494-551 lensTest, bsdfTest, capsuleTest, profileTest)
// on sm_103a, behind one C-ABI entry point (vt_unit_test). Each kernel runs one device function of the renderer on a
// caller's cases with the reference's input and output layout (float4 slots), so that the functions the path tracer
// inlines (the 8-step KB4 inverse, the BSDF lobes and their sampling, the albedo tables, the FDM layer normal, the
// capsule occlusion, the emission profile) can be checked one by one against a CPU restatement. traceTest is
// vt_trace_rays.
#include "vt_ctx.cuh"

namespace vtk {
using namespace vtd;
namespace {

constexpr int UT_THREADS = 64;   // the reference's @workgroup_size(64)

// lensTest: tin[i] = (u, v, -, -) is unprojected, tin[n + i] = (x, y, z, -) projected;
// tout[2i] = (ray, 0), tout[2i + 1] = (uv, 0, 0)
__global__ void lens_test_kernel(Kb4 L, const float4* __restrict__ in, float4* __restrict__ out, uint32_t n) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float4 a = in[i], b = in[n + i];
  const float3 r = kb4_unproject(L, a.x, a.y);
  const float2 uv = kb4_project(L, xyz(b));
  out[2 * i] = make_float4(r.x, r.y, r.z, 0.0f);
  out[2 * i + 1] = make_float4(uv.x, uv.y, 0.0f, 0.0f);
}

// bsdfTest: tin[4i..4i+3] = n, l, v, (u0, u1, u2, material); tout[3i] = (f, pdf(v -> l)), tout[3i + 1] = the
// sampled (l, pdf) or 0 when the sample is invalid, tout[3i + 2] = (albedoSpec(material, n.v), layerNormal(n,
// 0.1 l, normalize(v + (0.3, 0.1, 0.2)), 2e-4, 2e-5).x). A material index beyond the scene's gives NaN outputs.
__global__ void bsdf_test_kernel(const Scene S, uint32_t n_mat, const float4* __restrict__ in, float4* __restrict__ out, uint32_t n) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float3 nn = xyz(in[4 * i]), l = xyz(in[4 * i + 1]), v = xyz(in[4 * i + 2]);
  const float4 u = in[4 * i + 3];
  const uint32_t m = uint32_t(u.w);
  if (!(u.w >= 0.0f) || m >= n_mat) {
    const float q = __uint_as_float(0x7fc00000u);
    for (int k = 0; k < 3; k++) out[3 * i + k] = make_float4(q, q, q, q);
    return;
  }
  const Mat M = load_mat(S, m);
  const float3 f = eval_bsdf(M, nn, l, v);
  const float pdf = pdf_bsdf(M, nn, v, l);
  float3 ls = f3(0.0f, 0.0f, 0.0f);
  const float sp = sample_bsdf(M, nn, v, xyz(u), ls);
  const float3 a = albedo_part(S, M.idx, dot(nn, v), 0u);
  const float3 ln = layer_normal(nn, l * 0.1f, normalize(v + f3(0.3f, 0.1f, 0.2f)), 2e-4f, 2e-5f);
  out[3 * i] = make_float4(f.x, f.y, f.z, pdf);
  out[3 * i + 1] = sp > 0.0f ? make_float4(ls.x, ls.y, ls.z, sp) : make_float4(0.0f, 0.0f, 0.0f, 0.0f);
  out[3 * i + 2] = make_float4(a.x, a.y, a.z, ln.x);
}

// capsuleTest: tin[4i..4i+3] = p, n, (a, r), b; tout[i] = (capsuleOcc, 0, 0, 0)
__global__ void capsule_test_kernel(const float4* __restrict__ in, float4* __restrict__ out, uint32_t n) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float4 a = in[4 * i + 2];
  out[i] = make_float4(capsule_occ(xyz(in[4 * i]), xyz(in[4 * i + 1]), xyz(a), xyz(in[4 * i + 3]), a.w), 0.0f, 0.0f, 0.0f);
}

// profileTest: tin[i].x = theta; tout[i] = (p(theta), 0, 0, 0)
__global__ void profile_test_kernel(const Scene S, const float4* __restrict__ in, float4* __restrict__ out, uint32_t n) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  out[i] = make_float4(profile(S, in[i].x), 0.0f, 0.0f, 0.0f);
}

// float4 slots in and out per case of each kind
void unit_slots(uint32_t kind, uint32_t* in, uint32_t* out) {
  switch (kind) {
    case VT_UNIT_LENS: *in = 2; *out = 2; return;
    case VT_UNIT_BSDF: *in = 4; *out = 3; return;
    case VT_UNIT_CAPSULE: *in = 4; *out = 1; return;
    case VT_UNIT_PROFILE: *in = 1; *out = 1; return;
    default: *in = 0; *out = 0; return;
  }
}

}  // namespace
}  // namespace vtk

using namespace vtapi;

vt_status vt_unit_test(vt_ctx* ctx, const vt_unit_req* q, const float* in, float* out) {
  if (!ctx || !q) return VT_ERR_ARG;
  uint32_t si = 0, so = 0;
  vtk::unit_slots(q->kind, &si, &so);
  if (!si) return fail(ctx, VT_ERR_ARG, "unit test: unknown kind");
  if (!q->n) return VT_OK;
  if (!in || !out) return VT_ERR_ARG;
  if (q->n > (1u << 24)) return fail(ctx, VT_ERR_ARG, "unit test: at most 2^24 cases");
  vt_status s = reject_foreign(ctx, {in, out});
  if (s != VT_OK) return s;
  const size_t bin = size_t(q->n) * si * 16, bout = size_t(q->n) * so * 16;
  if ((s = ensure_scratch(ctx, (bin + 255) / 256 * 256 + bout + 256)) != VT_OK) return s;
  char* base = static_cast<char*>(ctx->d_scratch);
  float4* dIn = reinterpret_cast<float4*>(base);
  float4* dOut = reinterpret_cast<float4*>(base + (bin + 255) / 256 * 256);
  if ((s = to_device(ctx, dIn, in, bin)) != VT_OK) return s;
  const uint32_t blocks = (q->n + vtk::UT_THREADS - 1) / vtk::UT_THREADS;
  const vtd::Scene S = dev_scene(ctx);
  VT_CK(cudaEventRecord(ctx->ev0, ctx->stream));
  switch (q->kind) {
    case VT_UNIT_LENS: {
      // the reference's Lens: a = (fx, fy, cx, cy), b = (k1..k4), c = (alpha, -, -, -)
      const vtd::Kb4 L{q->lens[0], q->lens[1], q->lens[2], q->lens[3], q->lens[8], q->lens[4], q->lens[5], q->lens[6], q->lens[7]};
      vtk::lens_test_kernel<<<blocks, vtk::UT_THREADS, 0, ctx->stream>>>(L, dIn, dOut, q->n);
      break;
    }
    case VT_UNIT_BSDF:
      vtk::bsdf_test_kernel<<<blocks, vtk::UT_THREADS, 0, ctx->stream>>>(S, uint32_t(ctx->S.mats.size()), dIn, dOut, q->n);
      break;
    case VT_UNIT_CAPSULE:
      vtk::capsule_test_kernel<<<blocks, vtk::UT_THREADS, 0, ctx->stream>>>(dIn, dOut, q->n);
      break;
    default:
      vtk::profile_test_kernel<<<blocks, vtk::UT_THREADS, 0, ctx->stream>>>(S, dIn, dOut, q->n);
      break;
  }
  VT_CK(cudaGetLastError());
  VT_CK(cudaEventRecord(ctx->ev1, ctx->stream));
  ctx->tim.launches++;
  if ((s = from_device(ctx, out, dOut, bout)) != VT_OK) return s;
  VT_CK(cudaStreamSynchronize(ctx->stream));
  float ms = 0;
  cudaEventElapsedTime(&ms, ctx->ev0, ctx->ev1);
  ctx->tim.trace_ms = ms;
  return VT_OK;
}
