// C wrapper around the reference's OWN single-rank implementation — TEST INFRASTRUCTURE ONLY.
//
// Compiles the reference header src/pore_extraction.hpp unmodified (include path points at the
// read-only reference checkout; nothing is copied) against the project-written Kokkos shim in
// oracle/kokkos_compat/. The result, oracle/_ref/libpnm_ref*.so, pins the C restatement in
// oracle/pnm_oracle.c and generates the golden fixtures under tests/golden/. It is built only
// where the reference checkout exists and is never linked into the product.
//
// Argument conventions follow src/pnm_bindings.cpp after its zyx->xyz conversion: dims are
// (nx, ny, nz), origin/spacing are xyz float32, grad_p is xyz float64.
#include <cstdlib>
#include <cstring>
#include <vector>

#include "pore_extraction.hpp"

namespace {
template <class T>
T* dup(const std::vector<T>& v) {
  T* p = static_cast<T*>(std::malloc(sizeof(T) * (v.size() ? v.size() : 1)));
  if (!v.empty()) std::memcpy(p, v.data(), sizeof(T) * v.size());
  return p;
}
std::vector<float> vec(const float* p, std::size_t n) { return std::vector<float>(p, p + n); }
std::vector<double> vecd(const double* p, std::size_t n) {
  return p ? std::vector<double>(p, p + n) : std::vector<double>{};
}
}  // namespace

extern "C" {

struct ref_flow_result {
  long long n_pores, n_throats;
  float* pores;  // 4 * n_pores: x, y, z, radius
  double* pore_pressure;
  double* pore_residual;
  int* throats;  // 2 * n_throats
  double* throat_flow;
  double* throat_area;
  double* throat_dp;
};

void ref_free(void* p) { std::free(p); }

const char* ref_execution_space() { return Kokkos::DefaultExecutionSpace::name(); }

// pore_extraction.hpp:143 extract_pores_k
long long ref_extract_pores(const float* sdf, int nx, int ny, int nz, const float* org,
                            const float* spc, float** pores) {
  const std::size_t n = std::size_t(nx) * ny * nz;
  auto out = pnm::extract_pores_k(vec(sdf, n), {nx, ny, nz}, {org[0], org[1], org[2]},
                                  {spc[0], spc[1], spc[2]});
  std::vector<float> flat;
  for (auto& p : out) flat.insert(flat.end(), {p.x, p.y, p.z, p.radius});
  *pores = dup(flat);
  return (long long)out.size();
}

// pore_extraction.hpp:389 segment_volume_k
void ref_segment_volume(const float* sdf, int nx, int ny, int nz, const float* spc, int* seg) {
  const std::size_t n = std::size_t(nx) * ny * nz;
  auto s = pnm::segment_volume_k(vec(sdf, n), {nx, ny, nz}, {spc[0], spc[1], spc[2]});
  if (!s.empty()) std::memcpy(seg, s.data(), sizeof(int) * n);
}

// pore_extraction.hpp:157 segmentVolumeView with rootsOut: the gradient-path roots per voxel.
void ref_segment_with_roots(const float* sdf, int nx, int ny, int nz, const float* spc, int* seg,
                            int* roots) {
  const std::size_t n = std::size_t(nx) * ny * nz;
  if (!n) return;
  Kokkos::View<float*, pnm::Mem> d("sdf", n);
  pnm::uploadVec(vec(sdf, n), d);
  Kokkos::View<int*, pnm::Mem> r;
  auto s = pnm::segmentVolumeView(d, {nx, ny, nz}, {spc[0], spc[1], spc[2]}, &r);
  std::memcpy(seg, s.data(), sizeof(int) * n);
  std::memcpy(roots, r.data(), sizeof(int) * n);
}

// pore_extraction.hpp:454 extract_topology_k
long long ref_extract_topology(const int* seg, int nx, int ny, int nz, int** pairs) {
  const std::size_t n = std::size_t(nx) * ny * nz;
  auto c = pnm::extract_topology_k(std::vector<int>(seg, seg + n), {nx, ny, nz});
  std::vector<int> flat;
  for (auto& p : c) flat.insert(flat.end(), {p.first, p.second});
  *pairs = dup(flat);
  return (long long)c.size();
}

// pore_extraction.hpp:1011 extract_pore_network_k
void ref_extract_pore_network(const float* sdf, int nx, int ny, int nz, const float* org,
                              const float* spc, float** pores, long long* n_pores, int* seg,
                              int** pairs, long long* n_pairs) {
  const std::size_t n = std::size_t(nx) * ny * nz;
  auto net = pnm::extract_pore_network_k(vec(sdf, n), {nx, ny, nz}, {org[0], org[1], org[2]},
                                         {spc[0], spc[1], spc[2]});
  std::vector<float> pf;
  for (auto& p : net.pores) pf.insert(pf.end(), {p.x, p.y, p.z, p.radius});
  std::vector<int> cf;
  for (auto& p : net.connections) cf.insert(cf.end(), {p.first, p.second});
  *pores = dup(pf);
  *n_pores = (long long)net.pores.size();
  *pairs = dup(cf);
  *n_pairs = (long long)net.connections.size();
  if (!net.seg.empty()) std::memcpy(seg, net.seg.data(), sizeof(int) * n);
}

// pore_extraction.hpp:493 extract_network_flow_k. ox/oy/oz may be null (fully open grid).
ref_flow_result* ref_extract_network_flow(const float* sdf, int nx, int ny, int nz,
                                          const float* org, const float* spc, const double* u,
                                          const double* v, const double* w, const double* p,
                                          const double* ox, const double* oy, const double* oz,
                                          const double* grad_p) {
  const std::size_t n = std::size_t(nx) * ny * nz;
  pnm::NetworkFlow net;
  try {  // max label < 0 makes the reference size a view with a negative count (undefined)
    net = pnm::extract_network_flow_k(
      vec(sdf, n), {nx, ny, nz}, {org[0], org[1], org[2]}, {spc[0], spc[1], spc[2]}, vecd(u, n),
      vecd(v, n), vecd(w, n), vecd(p, n), vecd(ox, n), vecd(oy, n), vecd(oz, n),
      {grad_p[0], grad_p[1], grad_p[2]});
  } catch (...) {
    return nullptr;
  }
  auto* r = static_cast<ref_flow_result*>(std::calloc(1, sizeof(ref_flow_result)));
  r->n_pores = (long long)net.pores.size();
  r->n_throats = (long long)net.throats.size();
  std::vector<float> pf;
  for (auto& q : net.pores) pf.insert(pf.end(), {q.x, q.y, q.z, q.radius});
  std::vector<int> tf;
  for (auto& q : net.throats) tf.insert(tf.end(), {q.first, q.second});
  r->pores = dup(pf);
  r->pore_pressure = dup(net.pore_pressure);
  r->pore_residual = dup(net.pore_residual);
  r->throats = dup(tf);
  r->throat_flow = dup(net.throat_flow);
  r->throat_area = dup(net.throat_area);
  r->throat_dp = dup(net.throat_dp);
  return r;
}

void ref_flow_result_free(ref_flow_result* r) {
  if (!r) return;
  std::free(r->pores);
  std::free(r->pore_pressure);
  std::free(r->pore_residual);
  std::free(r->throats);
  std::free(r->throat_flow);
  std::free(r->throat_area);
  std::free(r->throat_dp);
  std::free(r);
}

}  // extern "C"
