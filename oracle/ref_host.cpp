// Host driver for the reference's own WGSL shaders, translated to C++ by
// oracle/wgsl2cpp.py into oracle/_ref/ref_shaders.inc.  TEST INFRASTRUCTURE
// ONLY (result checks and the CPU baseline); the product library never loads it.
//
// It restates the engine side of lbm-wgpu/src/lbm.rs that binds buffers and
// dispatches the shaders; the per-cell arithmetic is the reference's WGSL:
//   buffers      two sets of 9 f32 planes (create_data_buffers, lbm.rs:520-527,
//                lbm.rs:740-745), u32 barrier (lbm.rs:748-749), density_bg =
//                ux, uy, rho (lbm.rs:779-781), output (lbm.rs:782-784)
//   bind groups  pairs ne/sw = planes 2/6, nw/se = 0/8, n/s = 1/7, e/w = 5/3
//                (lbm.rs:760-771); the rest plane "origin" is set 0 plane 4
//                (lbm.rs:775)
//   dispatch     ceil(X*Y/256) workgroups of 256 invocations (lbm.rs:102-106)
//   step         collide = pre_corner, pre_cardinal, collide_corner,
//                collide_cardinal on set k%2; stream = e_w, n_s, nw_se, ne_sw
//                from set k%2 into set (k+1)%2 (lbm.rs:1112-1134, 1174-1252)
//   barrier      draw_barrier_updates with num_updates = 2*pairs - 1 and one
//                workgroup per pair (lbm.rs:1341-1356)
#include <cstdint>
#include <cstring>
#include <vector>
#include "_ref/ref_shaders.inc"

namespace {

struct RefLBM {
  uint32_t X, Y, N;
  float omega;
  uint64_t compute_step = 0;
  int threads = 1;
  std::vector<float> data[2][9];
  std::vector<uint32_t> barrier;
  std::vector<float> ux, uy, rho, output;
  std::vector<uint32_t> draw_points;
  uint32_t work_groups() const { return (N + 255u) / 256u; }
};

template <class T> wgsl::RArr<T> bind(std::vector<T>& v) {
  wgsl::RArr<T> a;
  a.p = v.data();
  a.n = (uint32_t)v.size();
  return a;
}

template <class F> void dispatch(RefLBM* s, F entry) {
  const long long total = (long long)s->work_groups() * 256;
#pragma omp parallel for num_threads(s->threads) schedule(static)
  for (long long g = 0; g < total; g++) entry(wgsl::uvec3{(uint32_t)g, 0u, 0u});
}

void pre_collide_corner(RefLBM* s) {
  auto& d = s->data[s->compute_step % 2];
  pre_corner::ne = bind(d[2]); pre_corner::sw = bind(d[6]);
  pre_corner::nw = bind(d[0]); pre_corner::se = bind(d[8]);
  pre_corner::ux = bind(s->ux); pre_corner::uy = bind(s->uy); pre_corner::rho = bind(s->rho);
  pre_corner::size = s->N;
  dispatch(s, pre_corner::entry);
}
void pre_collide_cardinal(RefLBM* s) {
  auto& d = s->data[s->compute_step % 2];
  pre_cardinal::n = bind(d[1]); pre_cardinal::s = bind(d[7]);
  pre_cardinal::e = bind(d[5]); pre_cardinal::w = bind(d[3]);
  pre_cardinal::ux = bind(s->ux); pre_cardinal::uy = bind(s->uy); pre_cardinal::rho = bind(s->rho);
  pre_cardinal::size = s->N;
  dispatch(s, pre_cardinal::entry);
}
void collide_corner_pass(RefLBM* s) {
  auto& d = s->data[s->compute_step % 2];
  collide_corner::ne = bind(d[2]); collide_corner::sw = bind(d[6]);
  collide_corner::nw = bind(d[0]); collide_corner::se = bind(d[8]);
  collide_corner::ux = bind(s->ux); collide_corner::uy = bind(s->uy); collide_corner::rho = bind(s->rho);
  collide_corner::size = s->N; collide_corner::omega = s->omega;
  collide_corner::origin = bind(s->data[0][4]);
  dispatch(s, collide_corner::entry);
}
void collide_cardinal_pass(RefLBM* s) {
  auto& d = s->data[s->compute_step % 2];
  collide_cardinal::n = bind(d[1]); collide_cardinal::s = bind(d[7]);
  collide_cardinal::e = bind(d[5]); collide_cardinal::w = bind(d[3]);
  collide_cardinal::ux = bind(s->ux); collide_cardinal::uy = bind(s->uy); collide_cardinal::rho = bind(s->rho);
  collide_cardinal::size = s->N; collide_cardinal::omega = s->omega;
  collide_cardinal::origin = bind(s->data[0][4]);
  dispatch(s, collide_cardinal::entry);
}

#define STREAM_PASS(fn, ns, A, B, ia, ib)                                   \
  void fn(RefLBM* s) {                                                      \
    auto& cur = s->data[s->compute_step % 2];                               \
    auto& nxt = s->data[(s->compute_step + 1) % 2];                         \
    ns::dimensions = ns::Dimensions{s->X, s->Y, s->N};                      \
    ns::A = bind(cur[ia]); ns::B = bind(cur[ib]);                           \
    ns::post_##A = bind(nxt[ia]); ns::post_##B = bind(nxt[ib]);             \
    ns::barrier = bind(s->barrier);                                         \
    dispatch(s, ns::entry);                                                 \
  }
STREAM_PASS(stream_e_w_pass, stream_e_w, e, w, 5, 3)
STREAM_PASS(stream_n_s_pass, stream_n_s, n, s, 1, 7)
STREAM_PASS(stream_nw_se_pass, stream_se_nw, nw, se, 0, 8)
STREAM_PASS(stream_ne_sw_pass, stream_ne_sw, ne, sw, 2, 6)

void compute_step(RefLBM* s) {
  pre_collide_corner(s);
  pre_collide_cardinal(s);
  collide_corner_pass(s);
  collide_cardinal_pass(s);
  stream_e_w_pass(s);
  stream_n_s_pass(s);
  stream_nw_se_pass(s);
  stream_ne_sw_pass(s);
  s->compute_step += 1;
}

}  // namespace

extern "C" {

typedef struct ref_sim ref_sim;

// LBM::new without the initial upload: the caller puts a state with
// ref_put_state; the barrier starts as init_barrier's two wall rows.
ref_sim* ref_create(uint32_t X, uint32_t Y, float omega) {
  if (X < 2 || Y < 2) return nullptr;
  RefLBM* s = new RefLBM();
  s->X = X; s->Y = Y; s->N = X * Y; s->omega = omega;
  for (int k = 0; k < 2; k++) for (int q = 0; q < 9; q++) s->data[k][q].assign(s->N, 0.0f);
  s->barrier.assign(s->N, 0u);
  for (uint32_t x = 0; x < X; x++) { s->barrier[x] = 1u; s->barrier[x + (Y - 1) * X] = 1u; }
  s->ux.assign(s->N, 0.0f); s->uy.assign(s->N, 0.0f); s->rho.assign(s->N, 0.0f);
  s->output.assign(s->N, 0.0f);
  s->draw_points.assign(2 * (size_t)s->N, 0u);
  return (ref_sim*)s;
}
void ref_destroy(ref_sim* h) { delete (RefLBM*)h; }
void ref_set_threads(ref_sim* h, int t) { ((RefLBM*)h)->threads = t < 1 ? 1 : t; }
void ref_set_omega(ref_sim* h, float w) { ((RefLBM*)h)->omega = w; }  // update_omega_buffer

// Uploads one state to both sets (as custom_speed / single_cell do) and
// restarts compute_step at 0.  pops9 is 9 planes of N floats, reference order.
void ref_put_state(ref_sim* h, const float* pops9) {
  RefLBM* s = (RefLBM*)h;
  for (int k = 0; k < 2; k++)
    for (int q = 0; q < 9; q++) std::memcpy(s->data[k][q].data(), pops9 + (size_t)q * s->N, s->N * 4);
  s->compute_step = 0;
}
void ref_set_barrier_buffer(ref_sim* h, const uint32_t* barrier) {
  RefLBM* s = (RefLBM*)h;
  std::memcpy(s->barrier.data(), barrier, s->N * 4);
}
void ref_get_barrier_buffer(ref_sim* h, uint32_t* barrier) {
  RefLBM* s = (RefLBM*)h;
  std::memcpy(barrier, s->barrier.data(), s->N * 4);
}
// draw_barrier_updates with (location, value) pairs.
void ref_draw_points(ref_sim* h, const uint32_t* pairs, uint32_t npairs) {
  RefLBM* s = (RefLBM*)h;
  if (npairs == 0 || npairs > s->N) return;
  std::memcpy(s->draw_points.data(), pairs, (size_t)npairs * 8);
  barrier_draw::num_updates = 2 * npairs - 1;
  barrier_draw::updates.p = reinterpret_cast<barrier_draw::Update*>(s->draw_points.data());
  barrier_draw::updates.n = s->N;
  barrier_draw::barrier = bind(s->barrier);
  for (uint32_t g = 0; g < npairs; g++) barrier_draw::entry(wgsl::uvec3{g, 0u, 0u});
}
void ref_iterate(ref_sim* h, uint64_t n) {
  RefLBM* s = (RefLBM*)h;
  for (uint64_t k = 0; k < n; k++) compute_step(s);
}
uint64_t ref_compute_step(ref_sim* h) { return ((RefLBM*)h)->compute_step; }

// Current populations (set compute_step%2, rest from set 0) and the density
// buffers (momenta ux, uy and rho) as float arrays.
void ref_get_state(ref_sim* h, float* pops9, float* rho, float* jx, float* jy) {
  RefLBM* s = (RefLBM*)h;
  const int cur = (int)(s->compute_step % 2);
  for (int q = 0; q < 9; q++) {
    const std::vector<float>& src = q == 4 ? s->data[0][4] : s->data[cur][q];
    if (pops9) std::memcpy(pops9 + (size_t)q * s->N, src.data(), s->N * 4);
  }
  if (rho) std::memcpy(rho, s->rho.data(), s->N * 4);
  if (jx) std::memcpy(jx, s->ux.data(), s->N * 4);
  if (jy) std::memcpy(jy, s->uy.data(), s->N * 4);
}
// Both sets, raw (set 0 then set 1, 9 planes each).
void ref_get_sets(ref_sim* h, float* set0, float* set1) {
  RefLBM* s = (RefLBM*)h;
  for (int q = 0; q < 9; q++) {
    std::memcpy(set0 + (size_t)q * s->N, s->data[0][q].data(), s->N * 4);
    std::memcpy(set1 + (size_t)q * s->N, s->data[1][q].data(), s->N * 4);
  }
}

// Summary statistics (lbm.rs:1051-1059): 0 curl, 1 ux, 2 uy, 3 rho, 4 speed.
void ref_summary(ref_sim* h, int stat, float* out) {
  RefLBM* s = (RefLBM*)h;
#define SUMMARY(ns)                                                   \
  ns::dimensions = ns::Dimensions{s->X, s->Y, s->N};                  \
  ns::ux = bind(s->ux); ns::uy = bind(s->uy); ns::rho = bind(s->rho); \
  ns::output = bind(s->output);                                       \
  dispatch(s, ns::entry);
  switch (stat) {
    case 0: { SUMMARY(sum_curl) break; }
    case 1: { SUMMARY(sum_ux) break; }
    case 2: { SUMMARY(sum_uy) break; }
    case 3: { SUMMARY(sum_rho) break; }
    case 4: { SUMMARY(sum_speed) break; }
    default: return;
  }
#undef SUMMARY
  std::memcpy(out, s->output.data(), s->N * 4);
}

// Colour map of the current output buffer (lbm.rs:1299-1335; ColorMap order
// 0 inferno, 1 viridis, 2 jet): rgb receives N * 3 floats.
void ref_color_map(ref_sim* h, int cmap, float* rgb) {
  RefLBM* s = (RefLBM*)h;
  std::vector<wgsl::vec3f> colors(s->N);
#define CMAP(ns)                                                        \
  ns::colors = bind(colors); ns::value = bind(s->output);               \
  ns::barrier = bind(s->barrier); ns::size = s->N;                      \
  dispatch(s, ns::entry);
  switch (cmap) {
    case 0: { CMAP(cmap_inferno) break; }
    case 1: { CMAP(cmap_viridis) break; }
    case 2: { CMAP(cmap_jet) break; }
    default: return;
  }
#undef CMAP
  for (uint32_t i = 0; i < s->N; i++) {
    rgb[3 * i] = colors[i].x;
    rgb[3 * i + 1] = colors[i].y;
    rgb[3 * i + 2] = colors[i].z;
  }
}

}  // extern "C"
