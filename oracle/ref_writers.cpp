/*
 * ref_writers.cpp -- TEST INFRASTRUCTURE ONLY.
 *
 * The reference host class's own output writers, compiled from the reference
 * tree (lbmcl.hpp:159-334: storeMap, storeF, storeData) against the OpenCL
 * stand-in in oracle/stub_cl, and exposed as C functions that write the
 * reference's files from host arrays (the oracle's data).  The digests of
 * those files (tests/golden/make_host_golden.py) pin the lbmcl host
 * program's output format to the reference's writers.  Built by
 * `make -C oracle refwriters` into oracle/_ref/; never part of the product.
 */
#include <cmath>
#include <cstring>
#include <fstream>
#include <iomanip>
#include <iostream>
#include <sstream>
#include <string>
#include <type_traits>
#include <utility>
#include <vector>

// the writers are private members of the reference class
#define private public
#include "lbmcl.hpp"
#undef private

namespace {

template <class T>
LBMCL<T> make(int dim, int iterations, int every, int stride, const char *vtk_path, const char *dump_path)
{
    // argument order of the reference constructor (lbmcl.hpp:338-352)
    return LBMCL<T>((size_t)dim, (T)0.0089, (T)0.05, (size_t)iterations, (size_t)every, vtk_path, 1, 1, 1,
                    (size_t)stride, false, dump_path, true, true);
}

template <class T> int store_f(int dim, int iterations, int stride, const T *f, int iteration, const char *path)
{
    LBMCL<T> L = make<T>(dim, iterations, 1, stride, "", path);
    std::vector<T> host((size_t)dim * dim * dim * Q);
    L.f_values = host.data();
    cl::Buffer b;
    b.host = f;
    L.storeF(b, (size_t)iteration);
    L.f_values = nullptr;
    return 0;
}

template <class T>
int store_data(int dim, int iterations, const T *rho, const T *u, int iteration, const char *vtk_path)
{
    LBMCL<T> L = make<T>(dim, iterations, 1, 32, vtk_path, "");
    std::vector<T> r((size_t)dim * dim * dim), v((size_t)3 * dim * dim * dim);
    L.rho_values = r.data();
    L.u_values = v.data();
    L.rho.host = rho;
    L.u.host = u;
    L.storeData((size_t)iteration);
    L.rho_values = nullptr;
    L.u_values = nullptr;
    return 0;
}

}  // namespace

extern "C" {

int refw_store_map(int dim, const int *map, const char *dump_path)
{
    LBMCL<float> L = make<float>(dim, 1, 1, 32, "", dump_path);
    std::vector<int> host((size_t)dim * dim * dim);
    L.map_values = host.data();
    L.map.host = map;
    L.storeMap();
    L.map_values = nullptr;
    return 0;
}

int refw_store_f_f32(int dim, int iterations, int stride, const float *f, int it, const char *path)
{
    return store_f<float>(dim, iterations, stride, f, it, path);
}
int refw_store_f_f64(int dim, int iterations, int stride, const double *f, int it, const char *path)
{
    return store_f<double>(dim, iterations, stride, f, it, path);
}
int refw_store_data_f32(int dim, int iterations, const float *rho, const float *u, int it, const char *path)
{
    return store_data<float>(dim, iterations, rho, u, it, path);
}
int refw_store_data_f64(int dim, int iterations, const double *rho, const double *u, int it, const char *path)
{
    return store_data<double>(dim, iterations, rho, u, it, path);
}

}  // extern "C"
