// lbmcl.hpp -- the LBMCL<T> host lattice class over the GB300 C ABI.
//
// Same public interface and outputs as the reference's class (lbmcl.hpp of
// LBMCL): the constructor arguments, setupSimulation / performSimulation /
// waitCompletion, the timing and MLUPS accessors, printConfiguration and
// statistics, and the map / f / ASCII VTI dump files.  The OpenCL objects are
// replaced by one lbm_t handle (include/lbm.h); nothing here touches CUDA.
//
// T is the type of the dumped values: float (FP32, FP16 and BF16 storage) or
// double (FP64 storage).
#pragma once

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <fstream>
#include <iomanip>
#include <iostream>
#include <sstream>
#include <stdexcept>
#include <string>
#include <type_traits>
#include <utility>
#include <vector>

#include "cell_types.h"
#include "lbm.h"

namespace lbmcl {

// number of decimal digits of val (lbmcl.hpp:13)
inline size_t digits(size_t val) { return val > 0 ? (size_t)std::log10((double)val) + 1 : 1; }

inline bool is_power_of_two(size_t x) { return x && !(x & (x - 1)); }

inline size_t previous_power_of_two(size_t x)
{
    size_t p = 1;
    while (p * 2 <= x) p *= 2;
    return x ? p : 0;
}

// A value as the reference passes it to its kernel build: printed with the
// stream's default 6 significant digits (lbmcl.hpp:140-141) and read back.
template <typename T> inline double as_kernel_literal(T v)
{
    std::ostringstream os;
    os << v;
    return std::strtod(os.str().c_str(), nullptr);
}

}  // namespace lbmcl

template <typename T>
class LBMCL
{
    static_assert(std::is_same<T, float>::value || std::is_same<T, double>::value,
                  "Only float or double data type is valid.");

    size_t dim;
    T viscosity;
    T velocity;
    size_t iterations;
    size_t every;
    std::string vtk_path;
    size_t lws[3];
    bool lws_given;
    size_t stride;
    bool optimize;
    std::string dump_path;
    bool dump_map;
    bool dump_f;
    bool dump_data;

    int storage;               // lbm_precision
    unsigned long long seed = 0;
    double noise = 0.0;
    int kernel = LBM_KERNEL_AUTO;
    bool binary = false;  // raw appended VTI and f_<it>.raw dumps
    int device = 0;

    lbm_t *h = nullptr;

    static void check(int rc)
    {
        if (rc != LBM_OK) {
            std::cerr << "lbm error " << rc << ": " << lbm_last_error() << std::endl;
            exit(rc);
        }
    }

    size_t n_sites() const { return dim * dim * dim; }
    size_t wet_dim() const { return (dim - 2) * (dim - 2) * (dim - 2); }
    size_t storage_bytes() const { return storage == LBM_FP64 ? 8 : (storage == LBM_FP32 ? 4 : 2); }
    size_t device_memory_size_b() const
    {
        const size_t n = n_sites();
        const size_t mb = storage == LBM_FP64 ? 8 : 4;
        return 2 * 19 * n * storage_bytes() + 4 * n * mb + n;
    }

    const char *storage_name() const
    {
        return storage == LBM_FP64 ? "fp64" : storage == LBM_FP32 ? "fp32" : storage == LBM_FP16 ? "fp16" : "bf16";
    }

    // map.dump (lbmcl.hpp:159-203)
    void storeMap()
    {
        std::vector<int32_t> m(n_sites());
        check(lbm_dump(h, LBM_DUMP_MAP, m.data(), m.size() * sizeof(int32_t)));
        std::ofstream out(dump_path + "/map.dump");
        out << "# FLUID       1\n# MOVING      2\n# BOUNDARY    3\n# WALL        4\n# CORNER      5\n\n";
        std::string line;
        for (size_t z = 0; z < dim; ++z) {
            for (size_t y = 0; y < dim; ++y) {
                line.clear();
                for (size_t x = 0; x < dim; ++x) {
                    line += std::to_string(lbmcl::cell_dump_code(m[x + y * dim + z * dim * dim]));
                    line += ' ';
                }
                out << line << '\n';
            }
            out << '\n';
        }
        out << '\n';
    }

    // f_<it>.dump (lbmcl.hpp:206-258): per (z, y) block a header row of q
    // indices, then per x "(x,y,z)" and the 19 values in fixed notation with 6
    // decimals in 8 columns; values de-indexed from the CSoA layout.
    void storeF(size_t iteration)
    {
        const size_t n = n_sites();
        std::vector<T> f(19 * n);
        check(lbm_dump(h, LBM_DUMP_F, f.data(), f.size() * sizeof(T)));
        std::ostringstream name;
        name << dump_path << "/f_" << std::setw((int)lbmcl::digits(iterations)) << std::setfill('0') << iteration
             << (binary ? ".raw" : ".dump");
        if (binary) {
            // the f buffer as the device holds it in the reference's layout:
            // 19 * dim^3 little-endian values in the CSoA order of `stride`
            std::ofstream raw(name.str(), std::ios::binary);
            raw.write(reinterpret_cast<const char *>(f.data()), (std::streamsize)(f.size() * sizeof(T)));
            return;
        }
        std::ofstream out(name.str());
        const size_t dd = lbmcl::digits(dim);
        const size_t coord_spaces = dd * 3 + 5;
        std::string head(coord_spaces, ' ');
        char buf[64];
        for (size_t q = 0; q < 19; ++q) {
            snprintf(buf, sizeof buf, "%8zu ", q);
            head += buf;
        }
        const size_t smask = stride - 1;
        std::string line;
        for (size_t z = 0; z < dim; ++z) {
            for (size_t y = 0; y < dim; ++y) {
                out << head << '\n';
                for (size_t x = 0; x < dim; ++x) {
                    const size_t id = x + y * dim + z * dim * dim;
                    snprintf(buf, sizeof buf, "%*s%zu,%zu,%zu) ", (int)dd, "(", x, y, z);
                    line = buf;
                    for (size_t q = 0; q < 19; ++q) {
                        const size_t k = ((id / stride) * 19 + q) * stride + (id & smask);
                        snprintf(buf, sizeof buf, "%8.6f ", (double)f[k]);
                        line += buf;
                    }
                    out << line << '\n';
                }
                out << '\n';
            }
            out << '\n';
        }
        out << '\n';
    }

    // lbmcl.<it>.vti with raw appended data: the same ImageData, extent and
    // arrays as the ASCII file; each array is a UInt64 byte count followed by
    // its values (rho, then v with the three components interleaved)
    void storeDataBinary(const std::string &path, const std::vector<T> &rho, const std::vector<T> &u)
    {
        const size_t n = n_sites();
        const size_t from = 1, to = dim - 1, extent = to - from - 1, m = dim - 2;
        const size_t npts = m * m * m;
        std::vector<T> r(npts), v(3 * npts);
        size_t k = 0;
        for (size_t z = from; z < to; ++z)
            for (size_t y = from; y < to; ++y)
                for (size_t x = from; x < to; ++x, ++k) {
                    const size_t id = x + y * dim + z * dim * dim;
                    r[k] = rho[id];
                    for (size_t c = 0; c < 3; ++c) v[3 * k + c] = u[c * n + id];
                }
        const uint64_t rb = npts * sizeof(T), vb = 3 * npts * sizeof(T);
        const char *type = std::is_same<T, float>::value ? "Float32" : "Float64";
        std::ofstream out(path, std::ios::binary);
        out << "<?xml version=\"1.0\"?>\n"
            << "<VTKFile type=\"ImageData\" version=\"0.1\" byte_order=\"LittleEndian\" header_type=\"UInt64\">\n"
            << "  <ImageData WholeExtent=\"0 " << extent << " 0 " << extent << " 0 " << extent
            << "\" Origin=\"0 0 0\" Spacing=\"1 1 1\">\n"
            << "    <Piece Extent=\"0 " << extent << " 0 " << extent << " 0 " << extent << "\">\n"
            << "      <PointData Scalars=\"rho\">\n"
            << "        <DataArray type=\"" << type
            << "\" Name=\"rho\" NumberOfComponents=\"1\" format=\"appended\" offset=\"0\"/>\n"
            << "        <DataArray type=\"" << type << "\" Name=\"v\" NumberOfComponents=\"3\" format=\"appended\" offset=\""
            << (sizeof(uint64_t) + rb) << "\"/>\n"
            << "      </PointData>\n"
            << "    </Piece>\n"
            << "  </ImageData>\n"
            << "  <AppendedData encoding=\"raw\">\n   _";
        out.write(reinterpret_cast<const char *>(&rb), sizeof rb);
        out.write(reinterpret_cast<const char *>(r.data()), (std::streamsize)rb);
        out.write(reinterpret_cast<const char *>(&vb), sizeof vb);
        out.write(reinterpret_cast<const char *>(v.data()), (std::streamsize)vb);
        out << "\n  </AppendedData>\n</VTKFile>\n";
    }

    // lbmcl.<it>.vti, ASCII ImageData of the interior [1, dim-2]^3
    // (lbmcl.hpp:261-334); --format binary writes raw appended data instead
    void storeData(size_t iteration)
    {
        const size_t n = n_sites();
        std::vector<T> rho(n), u(3 * n);
        check(lbm_dump(h, LBM_DUMP_RHO, rho.data(), rho.size() * sizeof(T)));
        check(lbm_dump(h, LBM_DUMP_U, u.data(), u.size() * sizeof(T)));
        std::ostringstream name;
        name << vtk_path << "/lbmcl." << std::setw((int)lbmcl::digits(iterations)) << std::setfill('0') << iteration
             << ".vti";
        if (binary) {
            storeDataBinary(name.str(), rho, u);
            return;
        }
        std::ofstream out(name.str());
        const size_t from = 1, to = dim - 1, extent = to - from - 1;
        const char *type = std::is_same<T, float>::value ? "Float32" : "Float64";
        out << "<?xml version=\"1.0\"?>\n"
            << "<VTKFile type=\"ImageData\" version=\"0.1\" byte_order=\"LittleEndian\" header_type=\"UInt64\">\n"
            << "  <ImageData WholeExtent=\"0 " << extent << " 0 " << extent << " 0 " << extent
            << "\" Origin=\"0 0 0\" Spacing=\"1 1 1\">\n"
            << "    <Piece Extent=\"0 " << extent << " 0 " << extent << " 0 " << extent << "\">\n"
            << "      <PointData Scalars=\"rho\">\n"
            << "        <DataArray type=\"" << type << "\" Name=\"rho\" NumberOfComponents=\"1\" format=\"ascii\">\n";
        char buf[48];
        std::string line;
        for (size_t z = from; z < to; ++z)
            for (size_t y = from; y < to; ++y) {
                line.clear();
                for (size_t x = from; x < to; ++x) {
                    snprintf(buf, sizeof buf, "%.16e ", (double)rho[x + y * dim + z * dim * dim]);
                    line += buf;
                }
                out << line << '\n';
            }
        out << "        </DataArray>\n"
            << "        <DataArray type=\"" << type << "\" Name=\"v\" NumberOfComponents=\"3\" format=\"ascii\">\n";
        for (size_t z = from; z < to; ++z)
            for (size_t y = from; y < to; ++y) {
                line.clear();
                for (size_t x = from; x < to; ++x) {
                    const size_t id = x + y * dim + z * dim * dim;
                    for (size_t c = 0; c < 3; ++c) {
                        snprintf(buf, sizeof buf, "%.16e ", (double)u[c * n + id]);
                        line += buf;
                    }
                }
                out << line << '\n';
            }
        out << "        </DataArray>\n"
            << "      </PointData>\n"
            << "    </Piece>\n"
            << "  </ImageData>\n"
            << "</VTKFile>\n";
    }

public:
    // lbmcl.hpp:338-388: dim and stride round down to a power of two, a work
    // group larger than the lattice is refused.
    LBMCL(size_t dim, T viscosity, T velocity, size_t iterations, size_t every, std::string vtk_path = "",
          size_t lwx = 1, size_t lwy = 1, size_t lwz = 1, size_t stride = 32, bool optimize = true,
          std::string dump_path = "", bool dump_map = false, bool dump_f = false, bool lws_given = true,
          int storage = -1)
        : dim(dim), viscosity(viscosity), velocity(velocity), iterations(iterations), every(every),
          vtk_path(vtk_path), lws{lwx, lwy, lwz}, lws_given(lws_given), stride(stride), optimize(optimize),
          dump_path(dump_path), dump_map(dump_map), dump_f(dump_f)
    {
        this->storage = storage >= 0 ? storage : (std::is_same<T, double>::value ? LBM_FP64 : LBM_FP32);
        dump_data = (every != 0);
        if (!lbmcl::is_power_of_two(dim)) {
            this->dim = lbmcl::previous_power_of_two(dim);
            std::cout << "dim is rounded to the previous power of 2: " << this->dim << std::endl;
        }
        if (lws[0] == 0) lws[0] = 1;
        if (lws[1] == 0) lws[1] = 1;
        if (lws[2] == 0) lws[2] = 1;
        if (lws[0] * lws[1] * lws[2] > this->dim * this->dim * this->dim) {
            std::cerr << "Please enter a good work_group_size to run the simulation" << std::endl;
            exit(-1);
        }
        if (!lbmcl::is_power_of_two(this->stride)) {
            this->stride = lbmcl::previous_power_of_two(this->stride);
            std::cout << "stride is rounded to the previous power of 2: " << this->stride << std::endl;
        }
    }

    ~LBMCL() { lbm_destroy(h); }

    LBMCL(const LBMCL &) = delete;
    LBMCL &operator=(const LBMCL &) = delete;

    void setNoise(unsigned long long s, double sigma) { seed = s; noise = sigma; }
    void setKernel(int k) { kernel = k; }
    void setBinary(bool b) { binary = b; }

    // lbmcl.hpp:392-482 + the initialize enqueue (lbmcl.hpp:494-498): one
    // handle owns every buffer; lbm_init also runs the initialisation kernel.
    void setupSimulation(int /*platformID*/, int deviceID)
    {
        device = deviceID < 0 ? 0 : deviceID;
        lbm_config c;
        lbm_config_default(&c);
        c.dim = (int)dim;
        c.viscosity = lbmcl::as_kernel_literal(viscosity);
        c.velocity = lbmcl::as_kernel_literal(velocity);
        c.precision = storage;
        c.stride = (int)stride;
        c.block_threads = lws_given ? (int)std::min<size_t>(1024, lws[0] * lws[1] * lws[2]) : 0;
        c.seed = seed;
        c.noise_sigma = noise;
        c.device = device;
        c.kernel = kernel;
        check(lbm_init(&h, &c));
    }

    // lbmcl.hpp:490-521 with the same file labels: f_<it> holds the buffer
    // iteration `it` reads, lbmcl.<it>.vti the moments iteration `it` stored.
    // Without dumps, the iterations are enqueued as one batch.
    void performSimulation()
    {
        if (dump_map) storeMap();
        if (dump_data) storeData(0);
        if (dump_f) storeF(0);
        size_t it = 1;
        while (it <= iterations) {
            size_t n = iterations - it + 1;
            if (dump_f) n = 1;
            else if (dump_data) n = std::min(n, every - ((it - 1) % every));  // up to the next output iteration
            if (dump_f) storeF(it);
            check(lbm_step(h, (int)n, (int)every));
            it += n;
            const size_t last = it - 1;
            if (dump_data && last % every == 0) storeData(last);
        }
    }

    void waitCompletion() { check(lbm_sync(h)); }

    void performSimulationAndWait()
    {
        performSimulation();
        waitCompletion();
    }

    // lbmcl.hpp:548-556: initialisation start to the end of the last work
    double totalTimeMS()
    {
        waitCompletion();
        double total = 0, kernels = 0;
        check(lbm_timing(h, &total, &kernels));
        return total;
    }

    // lbmcl.hpp:562-574: time of the iteration kernels only
    double kernelsTimeMS()
    {
        waitCompletion();
        double total = 0, kernels = 0;
        check(lbm_timing(h, &total, &kernels));
        return kernels;
    }

    // lbmcl.hpp:604-620
    double MLUPS() { return (wet_dim() * iterations) / (totalTimeMS() * 1000); }
    double kernelsMLUPS() { return (wet_dim() * iterations) / (kernelsTimeMS() * 1000); }

    std::string deviceName() const { return h ? lbm_device_name(h) : std::string("(not set up)"); }

    std::string kernelOptionsStr() const
    {
        std::ostringstream os;
        os << "DIM=" << dim << " STRIDE=" << stride << " VISCOSITY=" << viscosity << " VELOCITY=" << velocity
           << " STORAGE=" << storage_name() << " (run-time arguments, sm_103a)";
        return os.str();
    }

    // lbmcl.hpp:623-645
    void printConfiguration()
    {
        const std::string prec = std::is_same<T, float>::value ? "single" : "double";
        std::cout << std::boolalpha << "kernel options   = " << kernelOptionsStr() << "\n"
                  << "device           = " << deviceName() << "\n"
                  << "dim              = " << dim << "\n"
                  << "viscosity        = " << viscosity << "\n"
                  << "velocity         = " << velocity << "\n"
                  << "Device Mem. (B)  = " << device_memory_size_b() << "\n"
                  << "Device Mem. (KB) = " << device_memory_size_b() / (1 << 10) << "\n"
                  << "Device Mem. (MB) = " << device_memory_size_b() / (1 << 20) << "\n"
                  << "iterations       = " << iterations << "\n"
                  << "work_group_size  = (" << lws[0] << ", " << lws[1] << ", " << lws[2] << ")\n"
                  << "stride           = " << stride << "\n"
                  << "precision        = " << prec << "\n"
                  << "storage          = " << storage_name() << "\n"
                  << "optimize         = " << optimize << "\n"
                  << "every            = " << every << "\n"
                  << "VTK PATH         = " << vtk_path << "\n"
                  << "DUMP F           = " << dump_f << "\n"
                  << "DUMP MAP         = " << dump_map << "\n"
                  << "FORMAT           = " << (binary ? "binary" : "ascii") << "\n";
    }

    // lbmcl.hpp:648-669: the ';'-separated line benchmark.sh aggregates
    std::string statistics(char separator)
    {
        const std::string prec = std::is_same<T, float>::value ? "single" : "double";
        std::stringstream stat;
        stat << deviceName() << separator << prec << separator << dim << separator << iterations << separator
             << every << separator << std::setw(3) << std::setfill('0') << lws[0] << "," << std::setw(3)
             << std::setfill('0') << lws[1] << "," << std::setw(3) << std::setfill('0') << lws[2] << separator
             << stride << separator << optimize << separator << totalTimeMS() << separator << kernelsTimeMS()
             << separator << MLUPS() << separator << kernelsMLUPS() << "\n";
        return stat.str();
    }
};
