// VTK_Common.hpp -- legacy-format VTK writer of one subdomain's cell fields,
// the file layout of the reference's VTK output (src/libvis/VTK_Common.cpp:9-19,
// src/libvis/CLbmVisualizationVTK.hpp:27-99): ASCII STRUCTURED_GRID with the
// (imax+1)(jmax+1)(kmax+1) point coordinates, then CELL_DATA density (float),
// flag (INT) and velocity (float vectors), numbers printed with %f / %i.
//
// Formatting the text is the expensive part (tens of bytes per value); the
// ranges of each section are formatted in parallel by host threads into
// separate buffers and written in order, so the output is byte-identical to
// a serial fprintf loop.
#ifndef LBM_GB300_VTK_COMMON_HPP
#define LBM_GB300_VTK_COMMON_HPP

#include <algorithm>
#include <cstdio>
#include <functional>
#include <string>
#include <thread>
#include <vector>

#include "CVector.hpp"

namespace lbm_vtk {

// Appends the text of items [b, e) made by fmt(i, buf) (returns chars).
inline void format_range(std::string &out, size_t b, size_t e, const std::function<int(size_t, char *)> &fmt) {
    char buf[160];
    out.clear();
    out.reserve((e - b) * 12);
    for (size_t i = b; i < e; i++) out.append(buf, (size_t)fmt(i, buf));
}

// Formats n items with `threads` host threads and writes them in order.
inline bool write_items(FILE *fp, size_t n, unsigned threads, const std::function<int(size_t, char *)> &fmt) {
    if (n == 0) return true;
    threads = std::max(1u, std::min<unsigned>(threads, (unsigned)((n + 4095) / 4096)));
    const size_t block = (size_t)1 << 20;  // items per round, per thread at most
    std::vector<std::string> parts(threads);
    for (size_t base = 0; base < n; base += block * threads) {
        std::vector<std::thread> pool;
        const size_t span = std::min(n - base, block * threads);
        const size_t per = (span + threads - 1) / threads;
        for (unsigned t = 0; t < threads; t++) {
            const size_t b = base + std::min(span, t * per), e = base + std::min(span, (t + 1) * per);
            if (t + 1 == threads) format_range(parts[t], b, e, fmt);
            else pool.emplace_back([&, t, b, e] { format_range(parts[t], b, e, fmt); });
        }
        for (auto &th : pool) th.join();
        for (unsigned t = 0; t < threads; t++)
            if (!parts[t].empty() && fwrite(parts[t].data(), 1, parts[t].size(), fp) != parts[t].size()) return false;
    }
    return true;
}

// The reference's header (src/libvis/VTK_Common.cpp:9-19).
inline void write_vtkHeader(FILE *fp) {
    fprintf(fp, "# vtk DataFile Version 3.1\n");
    fprintf(fp, "Turbulent Fluid Simulation on MultiGPU.\n");
    fprintf(fp, "ASCII\n");
    fprintf(fp, "\n");
}

// One subdomain of imax x jmax x kmax cells of edge dx at origin_cell
// (cells), fields in x-fastest order: density[n], flags[n], velocity[3][n].
template <typename T>
bool write_vtk_cells(const char *path, int imax, int jmax, int kmax, T dx, CVector<3, int> origin_cell,
                     const T *density, const int *flags, const T *velocity, unsigned threads) {
    FILE *fp = fopen(path, "w");
    if (!fp) return false;
    const T ox = origin_cell[0] * dx, oy = origin_cell[1] * dx, oz = origin_cell[2] * dx;
    const size_t px = (size_t)imax + 1, py = (size_t)jmax + 1, pz = (size_t)kmax + 1;
    const size_t n = (size_t)imax * jmax * kmax;
    write_vtkHeader(fp);
    fprintf(fp, "DATASET STRUCTURED_GRID\n");
    fprintf(fp, "DIMENSIONS  %i %i %i \n", imax + 1, jmax + 1, kmax + 1);
    fprintf(fp, "POINTS %i float\n", (int)(px * py * pz));
    fprintf(fp, "\n");
    bool ok = write_items(fp, px * py * pz, threads, [&](size_t p, char *b) {
        const size_t i = p % px, j = (p / px) % py, k = p / (px * py);
        return snprintf(b, 160, "%f %f %f\n", (double)(ox + (T)i * dx), (double)(oy + (T)j * dx),
                        (double)(oz + (T)k * dx));
    });
    fprintf(fp, "\n");
    fprintf(fp, "CELL_DATA %i \n", (int)n);
    fprintf(fp, "SCALARS density float 1 \n");
    fprintf(fp, "LOOKUP_TABLE default \n");
    ok = ok && write_items(fp, n, threads, [&](size_t a, char *b) { return snprintf(b, 160, "%f\n", (double)density[a]); });
    fprintf(fp, "\n");
    fprintf(fp, "SCALARS flag INT 1 \n");
    fprintf(fp, "LOOKUP_TABLE default \n");
    ok = ok && write_items(fp, n, threads, [&](size_t a, char *b) { return snprintf(b, 160, "%i\n", flags[a]); });
    fprintf(fp, "\n");
    fprintf(fp, "VECTORS velocity float\n");
    ok = ok && write_items(fp, n, threads, [&](size_t a, char *b) {
        return snprintf(b, 160, "%f %f %f\n", (double)velocity[a], (double)velocity[n + a], (double)velocity[2 * n + a]);
    });
    return fclose(fp) == 0 && ok;
}

}  // namespace lbm_vtk

#endif
