// lbm_options.hpp -- command line of the lbmcl program.
//
// Same flags, defaults, validation messages and exit codes as the reference
// (lbm_options.hpp:32-196 of LBMCL): -P -D -d -n -u -i -e -v -w -s -F -o -p
// -m -f -h.  Long-only additions for this implementation: --precision
// (fp32|fp64|fp16|bf16), --seed, --noise, --kernel (auto|direct|narrow|staged),
// --format (ascii|binary: VTI with raw appended data and f_<it>.raw dumps).
#pragma once

#include <getopt.h>

#include <cstdio>
#include <cstdlib>
#include <iostream>
#include <limits>
#include <string>

#include "lbm.h"

#define LBMCL_RESULTS_FOLDER "./results"

struct lbm_options {
    int platformID = -1;
    int deviceID = -1;
    size_t dim = 8;
    double viscosity = 0.0089;
    double velocity = 0.05;
    size_t iterations = 10;
    size_t every = 1;
    std::string vtk_path = LBMCL_RESULTS_FOLDER;
    size_t lwx = 8, lwy = 8, lwz = 8;
    bool lws_given = false;
    size_t stride = 32;
    bool use_double = false;
    bool optimize = false;
    std::string dump_path = LBMCL_RESULTS_FOLDER;
    bool dump_map = false;
    bool dump_f = false;
    // additions
    int storage = -1;  // lbm_precision; -1: from -F (FP64) or FP32
    unsigned long long seed = 0;
    double noise = 0.0;
    int kernel = LBM_KERNEL_AUTO;
    bool binary = false;  // --format binary

    void print_help()
    {
        std::cout << "-P  --platform            Use the specified platform (accepted, CUDA has none)\n"
                     "-D  --device              Use the specified device                       \n"
                     "-d  --dim                 Set the lattice cube dimension                 \n"
                     "-n  --viscosity           Set the fluid viscosity                        \n"
                     "-u  --velocity            Set the x velocity of the moving wall          \n"
                     "-i  --iterations          Specify the number of iterations               \n"
                     "-e  --every               Save simulation results every N iterations     \n"
                     "-w  --work_group_size     Specify the work group size \"x,y,z\" (CUDA block = x*y*z threads)\n"
                     "-s  --stride              Specify the stride used in CSoA memory layout  \n"
                     "-F  --use_double          Make use of \"double\" type                    \n"
                     "-o  --optimize            Accepted; the CUDA kernels keep IEEE semantics \n"
                     "-v  --vtk_path            Specify where store VTI files                  \n"
                     "-p  --dump_path           Specify where store dumps                      \n"
                     "-m  --dump_map            Dump the lattice map                           \n"
                     "-f  --dump_f              Dump the lattice \"f\" for each iteration      \n"
                     "    --precision P         Population storage: fp32 fp64 fp16 bf16        \n"
                     "    --seed N              Seed of the initial noise                      \n"
                     "    --noise S             Std-dev of N(0,S^2) noise on FLUID populations \n"
                     "    --kernel K            Iteration kernel: auto direct narrow staged    \n"
                     "    --format F            Output files: ascii (default) or binary        \n"
                     "-h  --help                Show this help message and exit                \n";
        exit(1);
    }

    static int parse_int(const char *s)
    {
        try {
            return std::stoi(s);
        } catch (...) {
            return -1;
        }
    }

    void process_args(int argc, char *argv[])
    {
        opterr = 0;
        const char *const short_opts = "P:D:d:n:u:i:e:v:w:s:Fop:mfh";
        enum { OPT_PRECISION = 1000, OPT_SEED, OPT_NOISE, OPT_KERNEL, OPT_FORMAT };
        const option long_opts[] = {
            {"platform", required_argument, nullptr, 'P'},
            {"device", required_argument, nullptr, 'D'},
            {"dim", required_argument, nullptr, 'd'},
            {"viscosity", required_argument, nullptr, 'n'},
            {"velocity", required_argument, nullptr, 'u'},
            {"iterations", required_argument, nullptr, 'i'},
            {"every", optional_argument, nullptr, 'e'},
            {"work_group_size", optional_argument, nullptr, 'w'},
            {"stride", optional_argument, nullptr, 's'},
            {"use_double", no_argument, nullptr, 'F'},
            {"optimize", no_argument, nullptr, 'o'},
            {"vtk_path", optional_argument, nullptr, 'v'},
            {"dump_path", optional_argument, nullptr, 'p'},
            {"dump_map", no_argument, nullptr, 'm'},
            {"dump_f", no_argument, nullptr, 'f'},
            {"help", no_argument, nullptr, 'h'},
            {"precision", required_argument, nullptr, OPT_PRECISION},
            {"seed", required_argument, nullptr, OPT_SEED},
            {"noise", required_argument, nullptr, OPT_NOISE},
            {"kernel", required_argument, nullptr, OPT_KERNEL},
            {"format", required_argument, nullptr, OPT_FORMAT},
            {nullptr, no_argument, nullptr, 0},
        };

        int int_opt = -1;
        double real_opt = std::numeric_limits<double>::quiet_NaN();
        while (true) {
            const int opt = getopt_long(argc, argv, short_opts, long_opts, nullptr);
            if (opt < 0) break;
            switch (opt) {
            case 'P':
                if ((int_opt = parse_int(optarg)) < 0) { std::cerr << "Please enter a valid platform" << std::endl; exit(1); }
                platformID = int_opt;
                break;
            case 'D':
                if ((int_opt = parse_int(optarg)) < 0) { std::cerr << "Please enter a valid device" << std::endl; exit(1); }
                deviceID = int_opt;
                break;
            case 'd':
                if ((int_opt = parse_int(optarg)) < 0) { std::cerr << "Please enter a valid lattice dimension" << std::endl; exit(1); }
                dim = (size_t)int_opt;
                break;
            case 'n':
                if ((real_opt = std::atof(optarg)) < 0) { std::cerr << "Please enter a valid viscosity value" << std::endl; exit(1); }
                viscosity = real_opt;
                break;
            case 'u':
                velocity = std::atof(optarg);
                break;
            case 'i':
                if ((int_opt = parse_int(optarg)) < 0) { std::cerr << "Please enter a valid number of iterations" << std::endl; exit(1); }
                iterations = (size_t)int_opt;
                break;
            case 'e':
                if (!optarg || (int_opt = parse_int(optarg)) < 0) {
                    std::cerr << "Please enter a valid number for save simulation results every N iterations" << std::endl;
                    exit(1);
                }
                every = (size_t)int_opt;
                break;
            case 'w':
                if (optarg && sscanf(optarg, "%zu,%zu,%zu", &lwx, &lwy, &lwz) > 0) lws_given = true;
                break;
            case 's':
                if (!optarg || (int_opt = parse_int(optarg)) < 0) { std::cerr << "Please enter a valid number for stride value" << std::endl; exit(1); }
                stride = (size_t)int_opt;
                break;
            case 'F': use_double = true; break;
            case 'o': optimize = true; break;
            case 'v':
                vtk_path = optarg ? std::string(optarg) : std::string();
                if (vtk_path.empty()) {
                    vtk_path = LBMCL_RESULTS_FOLDER;
                    std::cout << "VTI files will be stored in:" << vtk_path << std::endl;
                }
                break;
            case 'p':
                dump_path = optarg ? std::string(optarg) : std::string();
                if (dump_path.empty()) {
                    dump_path = LBMCL_RESULTS_FOLDER;
                    std::cout << "dump files will be stored in: " << dump_path << std::endl;
                }
                break;
            case 'm': dump_map = true; break;
            case 'f': dump_f = true; break;
            case OPT_PRECISION: {
                const std::string p = optarg;
                if (p == "fp32") storage = LBM_FP32;
                else if (p == "fp64") storage = LBM_FP64;
                else if (p == "fp16") storage = LBM_FP16;
                else if (p == "bf16") storage = LBM_BF16;
                else { std::cerr << "Please enter a valid precision (fp32 fp64 fp16 bf16)" << std::endl; exit(1); }
                break;
            }
            case OPT_SEED: seed = std::strtoull(optarg, nullptr, 10); break;
            case OPT_NOISE:
                if ((real_opt = std::atof(optarg)) < 0) { std::cerr << "Please enter a valid noise value" << std::endl; exit(1); }
                noise = real_opt;
                break;
            case OPT_KERNEL: {
                const std::string k = optarg;
                if (k == "auto") kernel = LBM_KERNEL_AUTO;
                else if (k == "direct") kernel = LBM_KERNEL_DIRECT;
                else if (k == "narrow") kernel = LBM_KERNEL_NARROW;
                else if (k == "staged") kernel = LBM_KERNEL_STAGED;
                else { std::cerr << "Please enter a valid kernel (auto direct narrow staged)" << std::endl; exit(1); }
                break;
            }
            case OPT_FORMAT: {
                const std::string f = optarg;
                if (f == "ascii") binary = false;
                else if (f == "binary") binary = true;
                else { std::cerr << "Please enter a valid format (ascii binary)" << std::endl; exit(1); }
                break;
            }
            case 'h':
            case '?':
            default: print_help(); break;
            }
        }
    }

    // storage precision of the run: --precision wins over -F
    int precision() const { return storage >= 0 ? storage : (use_double ? LBM_FP64 : LBM_FP32); }
};
