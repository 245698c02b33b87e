// Drives the C++ shim (curvami-official_gb300/host/curvami_gb300.hpp) the way a C++ caller
// of the reference would: shape functions for faces and both sides of one fold, the
// assembler with the hinge, one deterministic assembly. Inputs and outputs are raw
// little-endian binary files written / read by tests/test_cpp_shim.py.
#include <cstdio>
#include <fstream>
#include <vector>

#include "../../curvami-official_gb300/host/curvami_gb300.hpp"

template <class T>
std::vector<T> read_vec(std::ifstream& f) {
  int64_t n = 0;
  f.read(reinterpret_cast<char*>(&n), 8);
  std::vector<T> v(n);
  f.read(reinterpret_cast<char*>(v.data()), n * sizeof(T));
  return v;
}

template <class T>
void write_vec(std::ofstream& f, const std::vector<T>& v) {
  const int64_t n = static_cast<int64_t>(v.size());
  f.write(reinterpret_cast<const char*>(&n), 8);
  f.write(reinterpret_cast<const char*>(v.data()), n * sizeof(T));
}

int main(int argc, char** argv) {
  if (argc != 3) return 2;
  std::ifstream in(argv[1], std::ios::binary);
  const auto nodes = read_vec<double>(in);
  const auto gp = read_vec<double>(in);
  const auto w = read_vec<double>(in);
  const auto crease = read_vec<double>(in);
  const auto left = read_vec<double>(in);
  const auto right = read_vec<double>(in);
  const auto fw = read_vec<double>(in);
  const auto ft = read_vec<double>(in);
  const auto x = read_vec<double>(in);
  const auto prm = read_vec<double>(in);  // rho, Kt, A(9), B(9), D(9)
  try {
    curvami_gb300::Context ctx(0);
    ctx.set_nodes(nodes);
    std::vector<curvami_gb300::Crease> cr(1);
    cr[0].xy = crease;
    cr[0].extend_start = cr[0].extend_end = true;
    auto faces = curvami_gb300::ShapeSet::build(ctx, gp, prm[0], 2, cr);
    auto L = curvami_gb300::ShapeSet::build(ctx, left, prm[0], 2, cr);
    auto R = curvami_gb300::ShapeSet::build(ctx, right, prm[0], 2, cr);
    std::vector<curvami_gb300::FoldSpec> folds(1);
    folds[0].left = &L;
    folds[0].right = &R;
    folds[0].weight = fw;
    folds[0].tangent = ft;
    folds[0].Kt = prm[1];
    curvami_gb300::NonLinearAssembler asm_(ctx, faces, w, folds);
    asm_.set_material(&prm[2], &prm[11], &prm[20]);
    std::vector<double> K, F;
    asm_.assemble(x, &K, F, CGB_TANGENT | CGB_HINGE | CGB_DETERMINISTIC);
    std::vector<int32_t> outer, inner;
    asm_.pattern(outer, inner);
    std::ofstream out(argv[2], std::ios::binary);
    write_vec(out, K);
    write_vec(out, F);
    write_vec(out, outer);
    write_vec(out, inner);
    std::printf("shim ok: nnz %lld\n", static_cast<long long>(asm_.nnz()));
  } catch (const curvami_gb300::Error& e) {
    std::fprintf(stderr, "error %d: %s\n", e.code, e.what());
    return 1;
  }
  return 0;
}
