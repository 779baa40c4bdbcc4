// io.cpp — output files of the mobility path in the reference's formats:
//   * a density on every sphere's grid, both poles added, as a VTK XML unstructured grid with one
//     piece per sphere and its parallel head (Sphere::writeVTU / writePVTU, Sphere/Sphere.cpp:322-365;
//     Shexp::writeVTU, Sphere/Shexp.cpp:96-204; grid with poles and cells as in
//     Shexp::getGridWithPole / getGridWithPoleCellConnect, :206-339). The pole values are the
//     density's spherical-harmonic expansion evaluated at theta = 1e-6 and pi - 1e-6 (the
//     reference's calcPoleValue, :382-405); the poles carry weight 0. File names follow the reference,
//     <prefix>Sphere_<name>_r0_<postfix>.vtu and <prefix>Sphere_<name>_<postfix>.pvtu, so its
//     result/Result2PVD.py collects them.
//   * sphere centres as XYZ (SphereSystem::writeXYZ, SRC/SphereSystem.cpp:158-179).
// Binary arrays use the VTK XML "binary" encoding: base64 of a UInt64 byte count followed by the
// little-endian data (the host is little endian on both supported platforms).
#include <cmath>
#include <complex>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <stdexcept>
#include <string>
#include <vector>

#include "../../include/smob.h"
#include "sh_host.h"
#include "smob_internal.h"

namespace smob {
void set_last_error(const char* msg);
}

namespace {

constexpr double kPi = 3.14159265358979323846264338327950288;

struct IoError : std::runtime_error {
    smob_status code;
    IoError(smob_status c, const std::string& m) : std::runtime_error(m), code(c) {}
};

template <typename F>
smob_status io_guard(F&& f) {
    try {
        return f();
    } catch (const IoError& e) {
        smob::set_last_error(e.what());
        return e.code;
    } catch (const std::exception& e) {
        smob::set_last_error(e.what());
        return SMOB_ERR_ARG;
    }
}

std::string base64_block(const void* data, size_t n) {
    static const char A[] = "ABCDEFGHIJKLMNOPQRSTUVWXYZabcdefghijklmnopqrstuvwxyz0123456789+/";
    std::vector<unsigned char> b(8 + n);
    const uint64_t len = n;
    std::memcpy(b.data(), &len, 8);
    if (n) std::memcpy(b.data() + 8, data, n);
    std::string out;
    out.reserve((b.size() + 2) / 3 * 4);
    for (size_t i = 0; i < b.size(); i += 3) {
        const uint32_t v = (uint32_t(b[i]) << 16) | (i + 1 < b.size() ? uint32_t(b[i + 1]) << 8 : 0u) |
                           (i + 2 < b.size() ? uint32_t(b[i + 2]) : 0u);
        out += A[(v >> 18) & 63];
        out += A[(v >> 12) & 63];
        out += i + 1 < b.size() ? A[(v >> 6) & 63] : '=';
        out += i + 2 < b.size() ? A[v & 63] : '=';
    }
    return out;
}

template <typename T>
void data_array(std::ofstream& f, const char* type, const std::string& name, int ncomp, const std::vector<T>& v) {
    f << "<DataArray type=\"" << type << "\" Name=\"" << name << "\" NumberOfComponents=\"" << ncomp
      << "\" format=\"binary\">\n"
      << base64_block(v.data(), v.size() * sizeof(T)) << "\n</DataArray>\n";
}

void qrot(const double* q, const double* v, double* o) {
    const double w = q[0], x = q[1], y = q[2], z = q[3];
    const double tx = 2 * (y * v[2] - z * v[1]);
    const double ty = 2 * (z * v[0] - x * v[2]);
    const double tz = 2 * (x * v[1] - y * v[0]);
    o[0] = v[0] + w * tx + (y * tz - z * ty);
    o[1] = v[1] + w * ty + (z * tx - x * tz);
    o[2] = v[2] + w * tz + (x * ty - y * tx);
}

// cells of the grid with poles (order p): point 0 = north pole, ring j point k = 1 + j(2p+2) + k,
// last point = south pole; triangles around the poles, quads between rings
void grid_cells(int p, std::vector<int32_t>& conn, std::vector<int32_t>& offs, std::vector<uint8_t>& types) {
    const int nphi = 2 * p + 2, south = (p + 1) * nphi + 1;
    auto id = [&](int j, int k) { return 1 + j * nphi + k; };
    auto cell = [&](std::initializer_list<int32_t> pts, uint8_t type) {
        conn.insert(conn.end(), pts);
        offs.push_back((int32_t)conn.size());
        types.push_back(type);
    };
    for (int k = 0; k < nphi; ++k) cell({0, id(0, k), id(0, (k + 1) % nphi)}, 5);  // VTK_TRIANGLE
    for (int j = 1; j <= p; ++j)
        for (int k = 0; k < nphi; ++k)
            cell({id(j, k), id(j, (k + 1) % nphi), id(j - 1, (k + 1) % nphi), id(j - 1, k)}, 9);  // VTK_QUAD
    cell({south, id(p, nphi - 1), id(p, 0)}, 5);
    for (int k = nphi - 2; k >= 0; --k) cell({south, id(p, k + 1), id(p, k)}, 5);
}

}  // namespace

extern "C" {

smob_status smob_write_vtu(smob_ctx* ctx, const char* prefix, const char* postfix, const char* name,
                           const double* density3m) {
    return io_guard([&]() -> smob_status {
        if (!ctx || !prefix || !postfix || !name || !density3m) throw IoError(SMOB_ERR_ARG, "null argument");
        const smob::HostSpheres h = smob::host_spheres(ctx);
        // spherical-harmonic coefficients of the density (body frame) for the pole values
        std::vector<int> off(h.N + 1);
        smob_status s = smob_coeff_offsets(ctx, off.data());
        if (s != SMOB_OK) return s;
        std::vector<double> coef(off[h.N]);
        s = smob_sh_g2s(ctx, density3m, coef.data());
        if (s != SMOB_OK) return s;

        const std::string piece = std::string("Sphere_") + name + "_r0_" + postfix + ".vtu";
        std::ofstream f(std::string(prefix) + piece, std::ios::out | std::ios::trunc);
        if (!f) throw IoError(SMOB_ERR_ARG, "cannot open " + std::string(prefix) + piece);
        f << "<?xml version=\"1.0\"?>\n<VTKFile type=\"UnstructuredGrid\" version=\"1.0\" "
             "byte_order=\"LittleEndian\" header_type=\"UInt64\">\n<UnstructuredGrid>\n";
        f.precision(17);
        for (int i = 0; i < h.N; ++i) {
            const int p = h.orders[i], nphi = 2 * p + 2, ng = (p + 1) * nphi, np = ng + 2;
            const double* q = h.quats + 4 * i;
            const double* c = h.centers + 3 * i;
            const double a = h.radii[i];
            const double zb[3] = {0, 0, 1};
            double z[3];
            qrot(q, zb, z);
            std::vector<double> pts(3 * np), val(3 * np), w(np, 0.0);
            const auto* ci = reinterpret_cast<const std::complex<double>*>(coef.data() + off[i]);
            double pole_b[3], pole[3];
            for (int pole_id = 0; pole_id < 2; ++pole_id) {
                const int at = pole_id == 0 ? 0 : np - 1;
                const double sgn = pole_id == 0 ? 1.0 : -1.0;
                smob::vsh_eval_point(p, ci, pole_id == 0 ? 1e-6 : kPi - 1e-6, 0.0, pole_b);
                qrot(q, pole_b, pole);
                for (int d = 0; d < 3; ++d) {
                    pts[3 * at + d] = c[d] + a * sgn * z[d];
                    val[3 * at + d] = pole[d];
                }
            }
            const int g0 = h.gidx[i];
            for (int k = 0; k < ng; ++k) {
                for (int d = 0; d < 3; ++d) {
                    pts[3 * (k + 1) + d] = h.coords[3 * (g0 + k) + d];
                    val[3 * (k + 1) + d] = density3m[3 * (g0 + k) + d];
                }
                w[k + 1] = h.weights[g0 + k];
            }
            std::vector<int32_t> conn, offs;
            std::vector<uint8_t> types;
            grid_cells(p, conn, offs, types);
            f << "<Piece NumberOfPoints=\"" << np << "\" NumberOfCells=\"" << types.size() << "\">\n";
            f << "<PointData Scalars=\"scalars\">\n";
            data_array(f, "Float64", name, 3, val);
            data_array(f, "Float64", "weights", 1, w);
            f << "</PointData>\n<Points>\n";
            data_array(f, "Float64", "points", 3, pts);
            f << "</Points>\n<Cells>\n";
            data_array(f, "Int32", "connectivity", 1, conn);
            data_array(f, "Int32", "offsets", 1, offs);
            data_array(f, "UInt8", "types", 1, types);
            f << "</Cells>\n</Piece>\n";
        }
        f << "</UnstructuredGrid>\n</VTKFile>\n";
        if (!f) throw IoError(SMOB_ERR_ARG, "write failed: " + std::string(prefix) + piece);

        const std::string head = std::string(prefix) + "Sphere_" + name + "_" + postfix + ".pvtu";
        std::ofstream ph(head, std::ios::out | std::ios::trunc);
        if (!ph) throw IoError(SMOB_ERR_ARG, "cannot open " + head);
        ph << "<?xml version=\"1.0\"?>\n<VTKFile type=\"PUnstructuredGrid\" version=\"1.0\" "
              "byte_order=\"LittleEndian\" header_type=\"UInt64\">\n<PUnstructuredGrid GhostLevel=\"0\">\n"
              "<PPointData Scalars=\"scalars\">\n"
           << "<PDataArray type=\"Float64\" Name=\"" << name << "\" NumberOfComponents=\"3\"/>\n"
           << "<PDataArray type=\"Float64\" Name=\"weights\" NumberOfComponents=\"1\"/>\n"
              "</PPointData>\n<PPoints>\n<PDataArray type=\"Float64\" Name=\"points\" NumberOfComponents=\"3\"/>\n"
              "</PPoints>\n"
           << "<Piece Source=\"" << piece << "\"/>\n</PUnstructuredGrid>\n</VTKFile>\n";
        if (!ph) throw IoError(SMOB_ERR_ARG, "write failed: " + head);
        return SMOB_OK;
    });
}

smob_status smob_write_xyz(smob_ctx* ctx, const char* path, const int* gids, double time) {
    return io_guard([&]() -> smob_status {
        if (!ctx || !path) throw IoError(SMOB_ERR_ARG, "null argument");
        const smob::HostSpheres h = smob::host_spheres(ctx);
        FILE* f = std::fopen(path, "w");
        if (!f) throw IoError(SMOB_ERR_ARG, "cannot open " + std::string(path));
        std::fprintf(f, "%d\n", h.N);
        std::fprintf(f, "SphereNumber: %d, time: %lf\n", h.N, time);
        for (int i = 0; i < h.N; ++i)
            std::fprintf(f, "S\t%d\t%.14g\t%.14g\t%.14g\t%.14g\n", gids ? gids[i] : i, h.radii[i], h.centers[3 * i],
                         h.centers[3 * i + 1], h.centers[3 * i + 2]);
        const bool ok = std::fclose(f) == 0;
        if (!ok) throw IoError(SMOB_ERR_ARG, "write failed: " + std::string(path));
        return SMOB_OK;
    });
}

}  // extern "C"
