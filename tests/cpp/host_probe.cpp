// host_probe.cpp -- test driver for the host-side C++ headers (no GPU):
//   host_probe conf <file>      parse conf.xml, print the fields
//   host_probe skeleton         CLbmSkeleton<float> of the reference defaults
//   host_probe vtk <file> <threads> <nx> <ny> <nz>   a VTK file of a synthetic subdomain
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <vector>

#include "lbm_gb300/CConfiguration.hpp"
#include "lbm_gb300/CLbmSkeleton.hpp"
#include "lbm_gb300/VTK_Common.hpp"

int main(int argc, char **argv) {
    if (argc >= 3 && !strcmp(argv[1], "conf")) {
        CConfiguration<float> c;
        try {
            c.loadFile(argv[2]);
        } catch (const char *m) {
            printf("error %s\n", m);
            return 3;
        }
        printf("viscosity %.9g\n", c.viscosity);
        printf("gravitation %.9g %.9g %.9g\n", c.gravitation[0], c.gravitation[1], c.gravitation[2]);
        printf("cavity %.9g %.9g %.9g %.9g\n", c.drivenCavityVelocity[0], c.drivenCavityVelocity[1],
               c.drivenCavityVelocity[2], c.drivenCavityVelocity[3]);
        printf("domain %d %d %d\n", c.domain_size[0], c.domain_size[1], c.domain_size[2]);
        printf("subdomains %d %d %d\n", c.subdomain_num[0], c.subdomain_num[1], c.subdomain_num[2]);
        printf("length %.9g %.9g %.9g\n", c.domain_length[0], c.domain_length[1], c.domain_length[2]);
        printf("loops %d\ntimestep %.9g\nvtk %d\nvalidate %d\n", c.loops, c.timestep, (int)c.do_visualization,
               (int)c.do_validate);
        printf("kernels %zu\ndevice %d\n", c.computation_kernel_count, c.device_nr);
        printf("lattice %d %.9g %.9g %.9g %.9g %s %llu %.9g\n", (int)c.lattice_units, c.lattice_tau,
               c.lattice_reynolds, c.lattice_lid, c.smagorinsky, c.storage.empty() ? "-" : c.storage.c_str(),
               c.seed, c.perturbation);
        return 0;
    }
    if (argc >= 2 && !strcmp(argv[1], "skeleton")) {
        // reference defaults: src/main.cpp:100-106, 32^3 cells of 0.1 m
        CVector<3, int> size(32, 32, 32), origin(0, 0, 0);
        CVector<3, float> len(0.1f, 0.1f, 0.1f), g(0, -9.81f, 0);
        CDomain<float> d(0, size, origin, len);
        CLbmSkeleton<float> s(d, CVector<4, float>(100, 0, 0, 1));
        s.init(g, 0.001308f, 1.0f);
        printf("tau %a\ninv_tau %a\ndt %a\ngravity %a %a %a\nlid %a\nre %a\nerror %d\n", s.tau, s.inv_tau,
               s.d_timestep, s.gravitation[0], s.gravitation[1], s.gravitation[2], s.drivenCavityVelocity[0],
               s.d_reynolds, (int)s.error());
        return 0;
    }
    if (argc >= 7 && !strcmp(argv[1], "vtk")) {
        const int nx = atoi(argv[4]), ny = atoi(argv[5]), nz = atoi(argv[6]), n = nx * ny * nz;
        std::vector<float> rho(n), vel(3 * n);
        std::vector<int> fl(n);
        for (int a = 0; a < n; a++) {
            rho[a] = 1.0f + 0.001f * (float)a - 0.0375f * (float)(a % 7);
            fl[a] = 1 << (a % 4);
            vel[a] = 0.01f * (float)((a * 37) % 101 - 50) / 7.0f;
            vel[n + a] = -0.02f * (float)(a % 5) / 3.0f;
            vel[2 * n + a] = 1e-7f * (float)a;
        }
        const bool ok = lbm_vtk::write_vtk_cells<float>(argv[2], nx, ny, nz, 0.1f / 32.0f, CVector<3, int>(2, 0, 6),
                                                        rho.data(), fl.data(), vel.data(), (unsigned)atoi(argv[3]));
        return ok ? 0 : 4;
    }
    return 1;
}
