// The whole OWM path of one cloud on the device, as the reference application
// runs it per loop iteration (CPP-TBB-CPU/application/owm_optim3.cpp:77-230):
// tree build, stage 1, sort + stage 2, LLP grid + stage 3, and the result
// (stage-3 ids followed by the LLPs).  Intermediates never leave the device;
// the host sees two small count words and the final seed list.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>

#include "owm_classes.cuh"
#include "owm_ctx.cuh"

namespace owm {

namespace {

__global__ void k_bbox(const double* __restrict__ xyz, int stride, int64_t n, long long* __restrict__ out) {
  long long x0 = 0x7FFFFFFFFFFFFFFFll, y0 = 0x7FFFFFFFFFFFFFFFll;
  long long x1 = (long long)0x8000000000000000ull, y1 = (long long)0x8000000000000000ull;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    long long x = dkey(xyz[stride * i]), y = dkey(xyz[stride * i + 1]);
    x0 = min(x0, x);
    x1 = max(x1, x);
    y0 = min(y0, y);
    y1 = max(y1, y);
  }
  for (int o = 16; o >= 1; o >>= 1) {
    x0 = min(x0, __shfl_xor_sync(0xffffffffu, x0, o));
    x1 = max(x1, __shfl_xor_sync(0xffffffffu, x1, o));
    y0 = min(y0, __shfl_xor_sync(0xffffffffu, y0, o));
    y1 = max(y1, __shfl_xor_sync(0xffffffffu, y1, o));
  }
  if ((threadIdx.x & 31) == 0) {
    atomicMin(out + 0, x0);
    atomicMin(out + 1, y0);
    atomicMax(out + 2, x1);
    atomicMax(out + 3, y1);
  }
}

// Plain x, y, z points into a cloud's 32-byte records (x, y, z, 0), each
// record written whole (two 16-byte stores), and its x, y array; and back.
__global__ void k_pad_points(const double* __restrict__ src, int64_t n, double* __restrict__ rec,
                             double* __restrict__ xy) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const double x = src[3 * i], y = src[3 * i + 1], z = src[3 * i + 2];
    double2* d = reinterpret_cast<double2*>(rec + 4 * i);
    d[0] = make_double2(x, y);
    d[1] = make_double2(z, 0.0);
    reinterpret_cast<double2*>(xy)[i] = make_double2(x, y);
  }
}

__global__ void k_unpad_points(const double* __restrict__ src, int64_t n, double* __restrict__ dst) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const double2* r = reinterpret_cast<const double2*>(src + 4 * i);
    const double2 a = r[0], b = r[1];
    dst[3 * i] = a.x;
    dst[3 * i + 1] = a.y;
    dst[3 * i + 2] = b.x;
  }
}

// seeds = s3[0..ns3) ++ llp[0..nllp) as int64 ids (-1 never occurs here).
__global__ void k_assemble(const uint32_t* __restrict__ s3, const uint32_t* __restrict__ ns3,
                           const uint32_t* __restrict__ llp, const uint32_t* __restrict__ nllp, int64_t cap,
                           int64_t* __restrict__ seeds) {
  const int64_t a = *ns3, b = *nllp;
  const int64_t tot = min(a + b, cap);
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < tot; i += (int64_t)gridDim.x * blockDim.x)
    seeds[i] = i < a ? (int64_t)s3[i] : (int64_t)llp[i - a];
}

size_t al(size_t b) { return (b + 255) & ~(size_t)255; }

}  // namespace

int clear_status(owm_ctx* c) {
  OWM_CUDA_TRY(cudaMemsetAsync(c->d_small + kStatusSlot, 0, 4, c->stream));
  return OWM_OK;
}

int check_input_status(owm_ctx* c) {
  OWM_CUDA_TRY(cudaMemcpyAsync(c->h_small + kStatusSlot, c->d_small + kStatusSlot, 4, cudaMemcpyDeviceToHost,
                               c->stream));
  OWM_CUDA_TRY(cudaStreamSynchronize(c->stream));
  uint32_t st = c->h_small[kStatusSlot];
  if (st & kStatusNonFinite) return OWM_EINVAL;
  if (st & kStatusWalkBound) return OWM_ETIMEOUT;
  return OWM_OK;
}

int device_bbox(owm_ctx* c, const double* d_xyz, int stride, int64_t n, owm_bbox* out) {
  long long init[4] = {0x7FFFFFFFFFFFFFFFll, 0x7FFFFFFFFFFFFFFFll, (long long)0x8000000000000000ull,
                       (long long)0x8000000000000000ull};
  long long* d = reinterpret_cast<long long*>(c->d_small + kBboxSlot);
  long long* h = reinterpret_cast<long long*>(c->h_small + kBboxSlot);
  std::memcpy(h, init, sizeof(init));
  OWM_CUDA_TRY(cudaMemcpyAsync(d, h, sizeof(init), cudaMemcpyHostToDevice, c->stream));
  int64_t g = std::min<int64_t>((n + 255) / 256, 152 * 8);
  const unsigned gb = (unsigned)std::max<int64_t>(g, 1);
  OWM_LAUNCH("k_bbox", c->stream, k_bbox<<<gb, 256, 0, c->stream>>>(d_xyz, stride, n, d));
  count_launch(&c->launches);
  OWM_CUDA_TRY(cudaMemcpyAsync(h, d, sizeof(init), cudaMemcpyDeviceToHost, c->stream));
  OWM_CUDA_TRY(cudaStreamSynchronize(c->stream));
  out->min_x = dkey_inv(h[0]);
  out->min_y = dkey_inv(h[1]);
  out->max_x = dkey_inv(h[2]);
  out->max_y = dkey_inv(h[3]);
  return OWM_OK;
}

int pad_points(const double* src, int64_t n, double* rec, double* xy, cudaStream_t s, int64_t* launches) {
  const unsigned g = (unsigned)std::max<int64_t>(1, std::min<int64_t>((n + 255) / 256, 152 * 16));
  OWM_LAUNCH("k_pad_points", s, k_pad_points<<<g, 256, 0, s>>>(src, n, rec, xy));
  count_launch(launches);
  OWM_CUDA_TRY(cudaGetLastError());
  return OWM_OK;
}

int unpad_points(const double* src, int64_t n, double* dst, cudaStream_t s, int64_t* launches) {
  const unsigned g = (unsigned)std::max<int64_t>(1, std::min<int64_t>((n + 255) / 256, 152 * 16));
  OWM_LAUNCH("k_unpad_points", s, k_unpad_points<<<g, 256, 0, s>>>(src, n, dst));
  count_launch(launches);
  OWM_CUDA_TRY(cudaGetLastError());
  return OWM_OK;
}

int run_stage1(owm_ctx* c, const TreeStore& t, const owm_params& p, Edge* ex, Edge* ey, uint32_t* d_win) {
  int rc = compute_edges(p, t.ox, t.oy, false, ex, ey, c->stream, &c->launches);
  if (rc) return rc;
  QueryJob j;
  j.tree = t.view(c->walk_limit);
  j.ex = ex;
  j.ey = ey;
  j.ncols = (int32_t)p.ncols;
  j.nrows = (int32_t)p.nrows;
  j.thr = p.min_num_points;
  j.cell_order = 0;
  j.patch_lx = patch_log2(c->tuning.walk_patch_x);
  j.skip = nullptr;
  j.out = d_win;
  j.status = c->d_small + kStatusSlot;
  j.warp_begin = 0;
  return run_query(j, c->d_job, c->stream, &c->launches, "k_query_s1");
}

int run_pipeline_enqueue(owm_ctx* c, const PointsView& pts, int64_t n, const owm_bbox& bb, const owm_run_cfg& cfg,
                         owm_params* p_out, int64_t** d_seeds, int64_t* room_out) {
  if (validate_tree_cfg(&cfg.tree) != OWM_OK) return OWM_EINVAL;
  owm_params& p = *p_out;
  int rc = owm_params_compute(&bb, n, cfg.wsize, cfg.overlap, cfg.bsize, &p);
  if (rc) return rc;
  const int64_t nc = p.ncells, ng = std::max<int64_t>(p.ngrid, 0);
  rc = tree_alloc(&c->tree, &c->tree_mem, n, cfg.tree, c->stream);
  if (rc) return rc;
  // scratch = [tree build | window classes | stage 2 | stage 3], disjoint:
  // the side stream zeroes stage 2's bitmaps and prepares stage 3's edge
  // tables while the tree is built, and runs stages 1-2 and stage 3's LLP
  // marks beside the hierarchy build.
  const size_t tbytes = (tree_scratch_bytes(n) + 255) & ~(size_t)255;
  const size_t cbytes = cfg.stage1_walk ? 0 : (classes_scratch_bytes(n, (int32_t)p.ncols, (int32_t)p.nrows) + 255) &
                                                  ~(size_t)255;
  const bool bitmap2 = p.overlap > 0.0;
  const size_t s2bytes = bitmap2 ? stage2_bitmap_scratch_bytes(n) : stage2_scratch_bytes(nc);
  const size_t s2al = (s2bytes + 255) & ~(size_t)255;
  size_t sbytes = tbytes + cbytes + s2al + stage3_scratch_bytes(ng);
  rc = c->scratch.reserve(sbytes, c->stream);
  if (rc) return rc;
  size_t obytes = 2 * al(65536 * sizeof(Edge)) + 2 * al((size_t)nc * 4) + al((size_t)std::max<int64_t>(ng, 1) * 4) +
                  al((size_t)(nc + ng + 1) * 8) + 1024;
  rc = c->outbuf.reserve(obytes, c->stream);
  if (rc) return rc;
  char* op = static_cast<char*>(c->outbuf.ptr);
  auto take = [&](size_t b) {
    void* q = op;
    op += al(b);
    return q;
  };
  Edge* ex = (Edge*)take(65536 * sizeof(Edge));
  Edge* ey = (Edge*)take(65536 * sizeof(Edge));
  uint32_t* win = (uint32_t*)take((size_t)nc * 4);
  uint32_t* llp = (uint32_t*)take((size_t)nc * 4);
  uint32_t* s3 = (uint32_t*)take((size_t)std::max<int64_t>(ng, 1) * 4);
  int64_t* s64 = (int64_t*)take((size_t)(nc + ng + 1) * 8);
  uint32_t* d_nllp = c->d_small + kLlpSlot;
  uint32_t* d_ns3 = c->d_small + kS3Slot;

  cudaStream_t s = c->stream;
  OWM_CUDA_TRY(cudaEventRecord(c->ev[0], s));
  rc = clear_status(c);
  ClassArgs cls;
  bool forked = false;
  if (!rc && !cfg.stage1_walk) {
    // Window edges and class tables, so that the build's gather can fold
    // every point into its window class on the fly.  They depend on nothing
    // the build makes before its gather, so they are prepared on the side
    // stream (forked after everything already queued on s, which may still
    // use this scratch) while the Morton pass and the sort run.
    cudaStream_t ss = c->side_stream;
    OWM_CUDA_TRY(cudaEventRecord(c->side_fork, s));
    OWM_CUDA_TRY(cudaStreamWaitEvent(ss, c->side_fork, 0));
    forked = true;
    rc = compute_edges(p, bb.min_x, bb.min_y, false, ex, ey, ss, &c->launches);
    if (!rc)
      rc = classes_prepare(p, ex, ey, static_cast<char*>(c->scratch.ptr) + tbytes, cbytes, n, &cls, ss, &c->launches);
    if (!rc && bitmap2)
      rc = stage2_bitmap_clear(static_cast<char*>(c->scratch.ptr) + tbytes + cbytes, s2al, n, ss);
    if (!rc)
      rc = run_stage3_prepare(bb.min_x, bb.min_y, p, static_cast<char*>(c->scratch.ptr) + tbytes + cbytes + s2al,
                              c->scratch.cap - tbytes - cbytes - s2al, ss, &c->launches);
    OWM_CUDA_TRY(cudaEventRecord(c->side_join, ss));
  }
  bool fused = false;
  c->stage12_side = false;
  c->tree.gather_block = c->tuning.gather_block;
  if (!rc)
    rc = build_tree(pts, n, bb, cfg.tree, &c->tree, c->scratch.ptr, tbytes, c->d_small + kStatusSlot, s,
                    &c->launches, cfg.stage1_walk ? nullptr : &cls, &fused, forked ? c->side_join : nullptr,
                    forked ? c->ev[6] : nullptr);
  void* s2scratch = static_cast<char*>(c->scratch.ptr) + tbytes + cbytes;
  const size_t s2cap = s2al;
  void* s3scratch = static_cast<char*>(c->scratch.ptr) + tbytes + cbytes + s2al;
  const size_t s3cap = c->scratch.cap - tbytes - cbytes - s2al;
  auto stage2 = [&](cudaStream_t st) {
    return bitmap2 ? run_stage2_bitmap(win, nc, n, p.overlap, llp, d_nllp, s2scratch, s2cap, st, &c->launches, forked)
                   : run_stage2(win, nc, n, p.overlap, llp, d_nllp, s2scratch, s2cap, st, &c->launches);
  };
  if (!rc && fused) {
    // The gather's class fold is all that stage 1 needs: finish stage 1,
    // run stage 2 and mark stage 3's LLP cells on the side stream (after its
    // table preparation and the gather) while s builds the hierarchy; join
    // before stage 3's queries.
    cudaStream_t ss = c->side_stream;
    c->stage12_side = true;
    OWM_CUDA_TRY(cudaStreamWaitEvent(ss, c->ev[6], 0));
    if (bitmap2) {  // the window kernel marks stage 2's bitmaps (zeroed early, above)
      uint32_t *once = nullptr, *twice = nullptr;
      stage2_bitmap_ptrs(s2scratch, n, &once, &twice);
      rc = classes_finish_marked(cls, p, win, once, twice, (uint32_t)n, ss, &c->launches);
    } else {
      rc = classes_finish(cls, c->tree.view(), n, p, win, ss, &c->launches);
    }
    if (!rc) OWM_CUDA_TRY(cudaEventRecord(c->ev[2], ss));
    if (!rc)
      rc = bitmap2 ? run_stage2_bitmap(win, nc, n, p.overlap, llp, d_nllp, s2scratch, s2cap, ss, &c->launches, true, true)
                   : stage2(ss);
    if (!rc) OWM_CUDA_TRY(cudaEventRecord(c->ev[3], ss));
    if (!rc) rc = run_stage3_mark(pts.xy, pts.xy_stride, p, llp, d_nllp, nc, s3scratch, s3cap, ss, &c->launches);
    OWM_CUDA_TRY(cudaEventRecord(c->side_join, ss));
  }
  // join (again, if the gather already did): nothing queued on s after this
  // point overtakes the side stream's work, on success or failure
  if (forked) OWM_CUDA_TRY(cudaEventRecord(c->ev[1], s));
  if (forked) OWM_CUDA_TRY(cudaStreamWaitEvent(s, c->side_join, 0));
  if (rc) return rc;
  if (c->stage12_side) {
    OWM_CUDA_TRY(cudaEventRecord(c->ev[7], s));
  } else {
    if (!forked) OWM_CUDA_TRY(cudaEventRecord(c->ev[1], s));
    if (cfg.stage1_walk) {
      rc = run_stage1(c, c->tree, p, ex, ey, win);
    } else {
      if (!fused) rc = classes_aggregate(cls, c->tree.view(), n, s, &c->launches);
      if (!rc) rc = classes_finish(cls, c->tree.view(), n, p, win, s, &c->launches);
    }
    if (rc) return rc;
    OWM_CUDA_TRY(cudaEventRecord(c->ev[2], s));
    rc = stage2(s);
    if (rc) return rc;
    OWM_CUDA_TRY(cudaEventRecord(c->ev[3], s));
  }
  rc = c->stage12_side
           ? run_stage3_query(c->tree.view(c->walk_limit, c->tuning.cell_warps), p, s3, d_ns3, s3scratch, s3cap, c->d_small + kStatusSlot, s, &c->launches)
           : run_stage3(c->tree.view(c->walk_limit, c->tuning.cell_warps), pts.xy, pts.xy_stride, p, llp, d_nllp, nc, s3, d_ns3, s3scratch, s3cap, c->d_job,
                        c->d_small + kStatusSlot, s, &c->launches);
  if (rc) return rc;
  OWM_CUDA_TRY(cudaEventRecord(c->ev[4], s));
  const int64_t room = nc + ng + 1;
  const unsigned ga = (unsigned)std::min<int64_t>((room + 255) / 256, 152 * 8);
  OWM_LAUNCH("k_assemble", s, k_assemble<<<ga, 256, 0, s>>>(s3, d_ns3, llp, d_nllp, room, s64));
  count_launch(&c->launches);
  OWM_CUDA_TRY(cudaGetLastError());
  *d_seeds = s64;
  *room_out = room;
  return OWM_OK;
}

int run_pipeline(owm_ctx* c, const PointsView& pts, int64_t n, const owm_bbox& bb, const owm_run_cfg& cfg,
                 int64_t* seeds, int64_t cap, int64_t* n_seeds, owm_run_info* info) {
  owm_params p;
  int64_t* s64 = nullptr;
  int64_t room = 0;
  int rc = run_pipeline_enqueue(c, pts, n, bb, cfg, &p, &s64, &room);
  if (rc) return rc;
  cudaStream_t s = c->stream;
  OWM_CUDA_TRY(cudaMemcpyAsync(c->h_small, c->d_small, 32, cudaMemcpyDeviceToHost, s));
  OWM_CUDA_TRY(cudaStreamSynchronize(s));
  if (c->h_small[kStatusSlot] & kStatusNonFinite) return OWM_EINVAL;
  if (c->h_small[kStatusSlot] & kStatusWalkBound) return OWM_ETIMEOUT;
  const int64_t nllp = c->h_small[kLlpSlot], ns3 = c->h_small[kS3Slot];
  const int64_t total = nllp + ns3;
  *n_seeds = total;
  if (info) {
    std::memset(info, 0, sizeof(*info));
    info->n_llp = nllp;
    info->n_stage3 = ns3;
    info->n_seeds = total;
    info->params = p;
  }
  if (total > cap) return OWM_ERANGE;
  if (total > 0) OWM_CUDA_TRY(cudaMemcpyAsync(seeds, s64, (size_t)total * 8, cudaMemcpyDefault, s));
  OWM_CUDA_TRY(cudaEventRecord(c->ev[5], s));
  OWM_CUDA_TRY(cudaStreamSynchronize(s));
  if (info) {
    // With stages 1-2 beside the hierarchy build, stage 1 counts from the
    // gather's end and stage 3 from the join, so the phases overlap.
    float a = 0, b = 0, d = 0, e = 0, f = 0;
    const bool side = c->stage12_side;
    cudaEventElapsedTime(&a, c->ev[0], c->ev[1]);
    cudaEventElapsedTime(&b, side ? c->ev[6] : c->ev[1], c->ev[2]);
    cudaEventElapsedTime(&d, c->ev[2], c->ev[3]);
    cudaEventElapsedTime(&e, side ? c->ev[7] : c->ev[3], c->ev[4]);
    cudaEventElapsedTime(&f, c->ev[0], c->ev[5]);
    info->ms_tree = a;
    info->ms_stage1 = b;
    info->ms_stage2 = d;
    info->ms_stage3 = e;
    info->ms_total = f;
  }
  return OWM_OK;
}

}  // namespace owm
