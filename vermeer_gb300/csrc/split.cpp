// split.cpp - one image rendered over several contexts (several GPUs).
//
// The reference parallelises a render over image tiles: each worker
// goroutine takes tiles from a channel and folds every pixel of a tile into
// the framebuffer (core/render.go:66-131, 184-204), so a pixel's running
// mean is only ever touched by one worker.  The split here keeps that
// property across devices: the image's rows are cut into one contiguous band
// per context, each context renders its band (vmr_render / vmr_render_path
// with row_begin/row_count, which samples every pixel exactly as the whole
// render does) on its own host thread and stream, straight into its rows of
// the caller's framebuffer.  No reduction is needed and the result is the
// one-context image bit for bit; the scene must have been loaded into every
// context identically (and, for a guided render, the guide's weights set
// alike).
#include <cstring>
#include <thread>
#include <vector>

#include "vmr.h"

namespace {

void stats_extra(vmr_render_stats& tot, const std::vector<vmr_render_stats>& st) {
  for (const auto& s : st) tot.camera_rays += s.camera_rays;
}
void stats_extra(vmr_path_stats& tot, const std::vector<vmr_path_stats>& st) {
  for (const auto& s : st) {
    tot.rays += s.rays;
    tot.graph_replays += s.graph_replays;
  }
}

template <class P, class S, class F>
int run_split(vmr_ctx* const* ctxs, uint32_t n, const P* p, float* fb, double* fb64, S* stats, F&& render_one) {
  if (!ctxs || n == 0 || !p || !fb || p->height == 0 || p->width == 0) return VMR_ERR_INVALID;
  if (p->row_count) return VMR_ERR_INVALID;  // the split makes the bands
  for (uint32_t i = 0; i < n; ++i)
    if (!ctxs[i]) return VMR_ERR_INVALID;
  std::vector<uint32_t> b(n), c(n);
  vmr_split_rows(p->height, n, b.data(), c.data());
  std::vector<int> rc(n, VMR_OK);
  std::vector<S> st(n);
  std::vector<std::thread> th;
  for (uint32_t i = 0; i < n; ++i) {
    if (c[i] == 0) continue;  // more contexts than rows
    th.emplace_back([&, i]() {
      P q = *p;
      q.row_begin = b[i];
      q.row_count = c[i];
      const size_t off = (size_t)b[i] * p->width * 3;
      rc[i] = render_one(ctxs[i], q, fb + off, fb64 ? fb64 + off : nullptr, &st[i]);
    });
  }
  for (auto& t : th) t.join();
  for (uint32_t i = 0; i < n; ++i)
    if (rc[i] != VMR_OK) return rc[i];
  if (stats) {
    S tot{};
    for (uint32_t i = 0; i < n; ++i) {
      tot.samples += st[i].samples;
      tot.shadow_rays += st[i].shadow_rays;
      if (st[i].ms > tot.ms) tot.ms = st[i].ms;  // the bands run at once: the slowest
    }
    stats_extra(tot, st);
    *stats = tot;
  }
  return VMR_OK;
}

}  // namespace

extern "C" {

int vmr_split_rows(uint32_t height, uint32_t n, uint32_t* row_begin, uint32_t* row_count) {
  if (n == 0 || !row_begin || !row_count) return VMR_ERR_INVALID;
  // bands of height / n rows, the first height % n of them one row taller
  const uint32_t q = height / n, r = height % n;
  uint32_t at = 0;
  for (uint32_t i = 0; i < n; ++i) {
    row_begin[i] = at;
    row_count[i] = q + (i < r ? 1u : 0u);
    at += row_count[i];
  }
  return VMR_OK;
}

int vmr_render_split(vmr_ctx* const* ctxs, uint32_t n, const vmr_render_params* p, float* fb,
                     vmr_render_stats* stats) {
  return run_split(ctxs, n, p, fb, nullptr, stats,
                   [](vmr_ctx* c, const vmr_render_params& q, float* f, double*, vmr_render_stats* s) {
                     return vmr_render(c, &q, f, s);
                   });
}

int vmr_render_path_split(vmr_ctx* const* ctxs, uint32_t n, const vmr_path_params* p, float* fb,
                          vmr_path_stats* stats) {
  if (p && (p->flags & VMR_PATH_TRAIN)) return VMR_ERR_UNSUPPORTED;
  return run_split(ctxs, n, p, fb, p ? p->fb64 : nullptr, stats,
                   [](vmr_ctx* c, const vmr_path_params& q, float* f, double* f64, vmr_path_stats* s) {
                     vmr_path_params r = q;
                     r.fb64 = f64;
                     return vmr_render_path(c, &r, f, s);
                   });
}

}  // extern "C"
