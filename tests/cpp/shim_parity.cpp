// C++ parity check of include/cgx_cabana.hpp: the reference-shaped p2g / g2p
// calls through libcgx against the FP64 oracle (liboracle). Built and run by
// tests/test_gpu_cpp_shim.py; prints "OK" and returns 0 on success.
#include <cuda_runtime.h>

#include <cmath>
#include <cstdint>
#include <cstdio>
#include <vector>

#include "../../oracle/cgx_oracle.hpp"
#include "cgx_cabana.hpp"

namespace {

uint64_t g_state = 0x9E3779B97F4A7C15ull;
double uniform01() {  // splitmix64
    uint64_t z = (g_state += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    z ^= z >> 31;
    return double(z >> 11) * (1.0 / 9007199254740992.0);
}

double max_rel(const std::vector<double>& a, const std::vector<double>& b) {
    double num = 0.0, den = 0.0;
    for (size_t i = 0; i < a.size(); ++i) {
        num = std::fmax(num, std::fabs(a[i] - b[i]));
        den = std::fmax(den, std::fabs(b[i]));
    }
    return den > 0.0 ? num / den : num;
}

template <class T>
T* to_device(const std::vector<T>& h) {
    T* d = nullptr;
    if (cudaMalloc(&d, h.size() * sizeof(T)) != cudaSuccess) return nullptr;
    cudaMemcpy(d, h.data(), h.size() * sizeof(T), cudaMemcpyHostToDevice);
    return d;
}

template <class T>
std::vector<T> to_host(const T* d, size_t n) {
    std::vector<T> h(n);
    cudaMemcpy(h.data(), d, n * sizeof(T), cudaMemcpyDeviceToHost);
    return h;
}

}  // namespace

int main() {
    namespace cc = cgx::cabana;
    const int cells = 16, n = 20000, order = 3;
    const double low[3] = {0.25, -1.0, 2.0}, h = 0.5;
    const int32_t owned[3] = {cells, cells, cells};
    const cc::LocalMesh lm = cc::LocalMesh::uniform(low, h, owned, 2);
    std::vector<double> pos(size_t(n) * 3), mass(n), mom(size_t(n) * 3);
    for (int p = 0; p < n; ++p) {
        for (int d = 0; d < 3; ++d) pos[size_t(p) * 3 + d] = low[d] + uniform01() * cells * h;
        mass[p] = 0.5 + uniform01();
        for (int d = 0; d < 3; ++d) mom[size_t(p) * 3 + d] = mass[p] * (2.0 * uniform01() - 1.0);
    }
    const int64_t nodes = lm.num_nodes();
    double* d_pos = to_device(pos);
    double* d_mass = to_device(mass);
    double* d_mom = to_device(mom);
    std::vector<double> zeros_m(nodes), zeros_p(size_t(nodes) * 3), zeros_v(size_t(n) * 3);
    double* d_mg = to_device(zeros_m);
    double* d_pg = to_device(zeros_p);
    double* d_vel = to_device(zeros_v);
    if (!d_pos || !d_mass || !d_mom || !d_mg || !d_pg || !d_vel) {
        std::printf("FAIL allocation\n");
        return 1;
    }
    auto points = cc::View<double, 2>::layout_right(d_pos, 3);
    auto mass_v = cc::View<double, 1>::layout_right(d_mass, 1);
    auto mom_v = cc::View<double, 2>::layout_right(d_mom, 3);
    auto vel_v = cc::View<double, 2>::layout_right(d_vel, 3);
    auto mass_g = cc::createArray(lm, 1, d_mg);
    auto mom_g = cc::createArray(lm, 3, d_pg);
    const cc::Halo halo = cc::createHalo(cc::NodeHaloPattern(), 2);
    try {
        cc::assign(mass_g, 0.0);
        cc::assign(mom_g, 0.0);
        cc::p2g(cc::createScalarValueP2G(mass_v, 1.0), points, n, cc::Spline<3>(), halo, mass_g);
        cc::p2g(cc::createVectorValueP2G(mom_v, -0.5), points, n, cc::Spline<3>(), halo, mom_g);
        cc::g2p(mom_g, halo, points, n, cc::Spline<3>(), cc::createVectorValueG2P(vel_v, 2.0));
    } catch (const std::exception& e) {
        std::printf("FAIL %s\n", e.what());
        return 1;
    }
    cudaDeviceSynchronize();
    // oracle
    oracle_mesh om;
    for (int d = 0; d < 3; ++d) {
        om.ghost_low[d] = lm.mesh.ghost_low[d];
        om.cell_size[d] = lm.mesh.cell_size[d];
        om.owned_cells[d] = lm.mesh.owned_cells[d];
        om.periodic[d] = 0;
    }
    om.halo_width = lm.mesh.halo_width;
    om.entity = 0;
    std::vector<double> mg(nodes, 0.0), pg(size_t(nodes) * 3, 0.0), vel(size_t(n) * 3, 0.0);
    oracle_op ops[2] = {{0, 1, 1.0, mass.data(), mg.data()}, {1, 3, -0.5, mom.data(), pg.data()}};
    oracle_p2g(&om, pos.data(), n, order, ops, 2, 1);
    oracle_op g[1] = {{1, 3, 2.0, vel.data(), pg.data()}};
    oracle_g2p(&om, pos.data(), n, order, g, 1, 1);
    const double e1 = max_rel(to_host(d_mg, nodes), mg);
    const double e2 = max_rel(to_host(d_pg, size_t(nodes) * 3), pg);
    const double e3 = max_rel(to_host(d_vel, size_t(n) * 3), vel);
    std::printf("errors %.3e %.3e %.3e\n", e1, e2, e3);
    // a rank mismatch does not compile; a NULL array surfaces as an exception
    bool threw = false;
    try {
        auto bad = cc::createArray<double>(lm, 1, nullptr);
        cc::p2g(cc::createScalarValueP2G(mass_v, 1.0), points, n, cc::Spline<3>(), halo, bad);
    } catch (const std::runtime_error&) {
        threw = true;
    }
    cudaFree(d_pos);
    cudaFree(d_mass);
    cudaFree(d_mom);
    cudaFree(d_mg);
    cudaFree(d_pg);
    cudaFree(d_vel);
    if (e1 > 1e-12 || e2 > 1e-12 || e3 > 1e-12 || !threw) {
        std::printf("FAIL\n");
        return 1;
    }
    std::printf("OK\n");
    return 0;
}
