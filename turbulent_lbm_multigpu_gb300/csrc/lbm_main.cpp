// lbm_main.cpp -- command-line driver with the reference's flags and modes
// (src/main.cpp:96-435) over the C++ interfaces of include/lbm_gb300/:
// normal runs and validate mode (decomposed domain against one domain of
// size global - 2*(n-1), velocity compared on rank 0's interior with the
// 1e-15 tolerance).  All subdomains run in this process on one GPU, so no
// MPI launcher is needed.  -u (unit tests) is accepted and does nothing:
// the reference registers no unit tests.
#include <getopt.h>
#include <unistd.h>

#include <cmath>
#include <cstdlib>
#include <cstring>
#include <iostream>
#include <list>
#include <string>
#include <vector>

#include "lbm_gb300/CManager.hpp"

typedef float T;
typedef Singleton<CConfiguration<T>> ConfigSingleton;

static void extract_comma_separated_integers(std::list<int> &out, const std::string &s) {
    size_t start = 0, comma;
    while ((comma = s.find(',', start)) != std::string::npos) {
        std::string sub = s.substr(start, comma - start);
        out.push_back(sub.empty() ? 0 : atoi(sub.c_str()));
        start = comma + 1;
    }
    out.push_back(atoi(s.substr(start).c_str()));
}

static int usage(const char *argv0) {
    std::cout << "usage: " << argv0 << std::endl
              << "\t\t[-x resolution_x, default: 32]\n\t\t[-y resolution_y, default: 32]\n"
              << "\t\t[-z resolution_z, default: 32]\n\t\t[-X subdomain resolution_x, default: 1]\n"
              << "\t\t[-Y subdomain resolution_y, default: 1]\n\t\t[-Z subdomain resolution_z, default: 1]\n\n"
              << "\t\t[-G gravitation in down direction, default: -9.81]\n\n"
              << "\t\t[-r viscosity, default: 0.001308]\n\t\t[-v]\t(debug mode on, be verbose)\n"
              << "\t\t[-d device_num]\n\t\t[-k number of kernels to run ]\n\t\t[-g]\t(VTK output flag)\n"
              << "\t\t[-R registers list]\t[-T work group threads list]\n"
              << "\t\t[-t timestep]\t(default: -1 for automatic detection)\n"
              << "    \t[-u] run unit tests\n    \t[-c] read the configuration file\n"
              << "    \t[-b] append the timing to output/benchmark/benchmark_<subdomains>.ini" << std::endl;
    return -1;
}

int main(int argc, char **argv) {
    bool debug = false;
    CVector<3, int> domain_size(32, 32, 32), subdomain_nums(1, 1, 1);
    CVector<3, T> domain_length(0.1f, 0.1f, 0.1f), gravitation(0, -9.81f, 0);
    CVector<4, T> cavity(100, 0, 0, 1);
    T viscosity = 0.001308f, timestep = -1.0f;
    int loops = -1, device_nr = 0;
    bool do_vis = false, unit_test = false, use_conf = false, benchmark = false;
    size_t kernel_count = 128;
    std::string regs, threads, conf_file;
    int ch;
    while ((ch = getopt(argc, argv, "x:y:z:d:vr:k:gG:t:sl:R:T:X:Y:Z:S:u:c:n:m:p:b")) > 0) {
        switch (ch) {
            case 'd': device_nr = atoi(optarg); break;
            case 'v': debug = true; break;
            case 'R': regs = optarg; break;
            case 'T': threads = optarg; break;
            case 'x': domain_size[0] = atoi(optarg); break;
            case 'y': domain_size[1] = atoi(optarg); break;
            case 'z': domain_size[2] = atoi(optarg); break;
            case 'X': subdomain_nums[0] = atoi(optarg); break;
            case 'Y': subdomain_nums[1] = atoi(optarg); break;
            case 'Z': subdomain_nums[2] = atoi(optarg); break;
            case 'S': domain_size = CVector<3, int>(atoi(optarg)); break;
            case 'l': loops = atoi(optarg); break;
            case 'k': kernel_count = atoi(optarg); break;
            case 'r': viscosity = atof(optarg); break;
            case 'n': domain_length[0] = atof(optarg); break;
            case 'm': domain_length[1] = atof(optarg); break;
            case 'p': domain_length[2] = atof(optarg); break;
            case 'g': do_vis = true; break;
            case 'G': gravitation[1] = atof(optarg); break;
            case 't': timestep = atof(optarg); break;
            case 's': break;
            case 'u': unit_test = true; break;
            case 'c': use_conf = true; conf_file = optarg; break;
            case 'b': benchmark = true; break;
            default: return usage(argv[0]);
        }
    }
    CConfiguration<T> *cfg = ConfigSingleton::Instance();
    try {
        if (use_conf) {
            cfg->loadFile(conf_file);
        } else {
            cfg->domain_size = domain_size;
            cfg->subdomain_num = subdomain_nums;
            cfg->domain_length = domain_length;
            cfg->gravitation = gravitation;
            cfg->viscosity = viscosity;
            cfg->computation_kernel_count = kernel_count;
            cfg->device_nr = device_nr;
            cfg->do_visualization = do_vis;
            cfg->timestep = timestep;
            cfg->loops = loops;
            cfg->drivenCavityVelocity = cavity;
            if (!threads.empty()) extract_comma_separated_integers(cfg->lbm_opencl_number_of_threads_list, threads);
            if (!regs.empty()) extract_comma_separated_integers(cfg->lbm_opencl_number_of_registers_list, regs);
        }
        cfg->debug_mode = debug;
        if (benchmark) cfg->benchmark = true;
        if (debug) cfg->printMe();
        if (unit_test) {
            std::cout << "no unit tests are registered" << std::endl;
            return 0;
        }
        CVector<3, int> origin(0, 0, 0);
        if (cfg->do_validate) {
            CDomain<T> domain(-1, cfg->domain_size, origin, cfg->domain_length);
            CManager<T> manager(domain, cfg->subdomain_num);
            manager.initSimulation(0);
            manager.startSimulation();
            CController<T> *ctl = manager.getController();
            CVector<3, int> with_halo = ctl->getDomain().getSize();
            CVector<3, int> local(with_halo[0] - 2, with_halo[1] - 2, with_halo[2] - 2), lo(1, 1, 1);
            std::vector<T> local_data((size_t)local.elements() * 3);
            ctl->getSolver()->storeVelocity(local_data.data(), lo, local);

            CVector<3, int> vsize(cfg->domain_size[0] - 2 * (cfg->subdomain_num[0] - 1),
                                  cfg->domain_size[1] - 2 * (cfg->subdomain_num[1] - 1),
                                  cfg->domain_size[2] - 2 * (cfg->subdomain_num[2] - 1));
            CVector<3, T> cell(cfg->domain_length[0] / (T)cfg->domain_size[0],
                               cfg->domain_length[1] / (T)cfg->domain_size[1],
                               cfg->domain_length[2] / (T)cfg->domain_size[2]);
            CVector<3, T> vlen(vsize[0] * cell[0], vsize[1] * cell[1], vsize[2] * cell[2]);
            CDomain<T> vdomain(-2, vsize, origin, vlen);
            CManager<T> vmanager(vdomain, CVector<3, int>(1, 1, 1));
            std::cout << "--> Compute the results for one domain." << std::endl;
            vmanager.initSimulation(-1);
            vmanager.startSimulation();
            std::vector<T> global((size_t)local.elements() * 3);
            CVector<3, int> so(1, 1, 1);  // rank 0 sits at the origin
            vmanager.getController()->getSolver()->storeVelocity(global.data(), so, local);
            const double tol = 1.0e-15;
            int errors = 0;
            for (size_t i = 0; i < global.size(); i++)
                if (std::fabs((double)global[i] - (double)local_data[i]) > tol) errors++;
            std::cout << "VALIDATION SIZE: " << vsize << std::endl;
            std::cout << "--> TOLERANCE: " << tol << " NUMBER OF FAILED CELLS/TOTAL NUMBER OF CELLS: " << errors << "/"
                      << local.elements() << std::endl;
            return errors == 0 ? 0 : 2;
        }
        CDomain<T> domain(-1, cfg->domain_size, origin, cfg->domain_length);
        CManager<T> manager(domain, cfg->subdomain_num);
        manager.initSimulation(0);
        manager.startSimulation();
        if (debug) {
            float checksum = manager.getController()->getSolver()->getVelocityChecksum();
            std::cout.precision(8);
            std::cout << "Checksum: " << std::fixed << (checksum * 1000.0f) << std::endl;
        }
    } catch (const char *msg) {
        std::cerr << "error: " << msg << std::endl;
        return 1;
    }
    return 0;
}
