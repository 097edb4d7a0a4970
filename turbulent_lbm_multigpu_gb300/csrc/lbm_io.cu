// lbm_io.cu -- checkpoint / restart of lattices and decomposed domains.
//
// A checkpoint holds the raw stored populations (the 19 planes exactly as
// they are in HBM: float, double, or the shifted 16-bit forms bit for bit)
// and the flag bytes of every lattice, with the step counter.  The counter's
// parity is the A-A slot layout of the stored populations (even: standard
// slots after a beta step or the initial state; odd: opposite slots after an
// alpha step), so a restart continues with the same kernel sequence and the
// results are bit-identical to an uninterrupted run.  No reference
// counterpart: the reference writes VTK snapshots only.
//
// File layout (little-endian):
//   lattice file: LatHeader, then the lattice block
//   domain file:  DomHeader, then one lattice block per subdomain in order
//   lattice block: flags (n bytes), then planes 0..18 (n elements each),
//                  then the FNV-1a 64 hash of those bytes.
// Data moves through a bounded pinned host buffer, plane by plane.
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "lbm_internal.h"

using namespace lbm;
using namespace lbm_rt;

namespace lbm_rt {

namespace {

constexpr char kLatMagic[8] = {'L', 'B', 'M', 'C', 'K', 'P', 'T', '1'};
constexpr size_t kChunk = (size_t)64 << 20;  // host staging: 64 MB (a multiple of 8)

struct LatHeader {
    char magic[8];
    int32_t storage;
    int32_t nx, ny, nz;
    int64_t counter;
};
static_assert(sizeof(LatHeader) == 32, "checkpoint header layout");

// FNV-1a over 64-bit little-endian words of each staged chunk (trailing
// bytes one by one); save and load stage the same chunks.
struct Fnv {
    uint64_t h = 1469598103934665603ull;
    void add(const unsigned char *p, size_t n) {
        size_t i = 0;
        for (; i + 8 <= n; i += 8) {
            uint64_t w = 0;
            for (int b = 0; b < 8; b++) w |= (uint64_t)p[i + b] << (8 * b);
            h = (h ^ w) * 1099511628211ull;
        }
        for (; i < n; i++) h = (h ^ p[i]) * 1099511628211ull;
    }
};

// Pinned staging buffer for the lifetime of one call.
struct Staging {
    unsigned char *p = nullptr;
    size_t n = 0;
    ~Staging() {
        if (p) cudaFreeHost(p);
    }
    int init(size_t bytes) {
        n = bytes;
        if (cudaMallocHost((void **)&p, n) != cudaSuccess) {
            p = nullptr;
            return fail("cudaMallocHost of the checkpoint staging buffer failed");
        }
        return 0;
    }
};

struct File {
    FILE *f = nullptr;
    ~File() {
        if (f) fclose(f);
    }
};

// Device -> file, `bytes` from `src`, through the staging buffer.
int write_region(FILE *f, const void *src, size_t bytes, Staging &sg, Fnv &h) {
    for (size_t o = 0; o < bytes; o += sg.n) {
        const size_t k = std::min(sg.n, bytes - o);
        CU(cudaMemcpy(sg.p, (const unsigned char *)src + o, k, cudaMemcpyDeviceToHost));
        h.add(sg.p, k);
        if (fwrite(sg.p, 1, k, f) != k) return fail("checkpoint write failed");
    }
    return 0;
}

// File -> device.
int read_region(FILE *f, void *dst, size_t bytes, Staging &sg, Fnv &h) {
    for (size_t o = 0; o < bytes; o += sg.n) {
        const size_t k = std::min(sg.n, bytes - o);
        if (fread(sg.p, 1, k, f) != k) return fail("checkpoint file is truncated");
        h.add(sg.p, k);
        CU(cudaMemcpy((unsigned char *)dst + o, sg.p, k, cudaMemcpyHostToDevice));
    }
    return 0;
}

}  // namespace

int ckpt_write_lattice(FILE *f, lbm_lattice *l, int64_t counter) {
    LatHeader hd{};
    memcpy(hd.magic, kLatMagic, 8);
    hd.storage = l->storage;
    hd.nx = l->nx; hd.ny = l->ny; hd.nz = l->nz;
    hd.counter = counter;
    if (fwrite(&hd, sizeof(hd), 1, f) != 1) return fail("checkpoint write failed");
    const size_t eb = storage_bytes(l->storage), pb = (size_t)l->n * eb;
    Staging sg;
    if (sg.init(std::min(kChunk, std::max(pb, (size_t)l->n)))) return -1;
    Fnv h;
    if (write_region(f, l->flags, (size_t)l->n, sg, h)) return -1;
    for (int i = 0; i < 19; i++)
        if (write_region(f, (const unsigned char *)l->dd + (size_t)i * l->pstride * eb, pb, sg, h)) return -1;
    if (fwrite(&h.h, sizeof(h.h), 1, f) != 1) return fail("checkpoint write failed");
    return 0;
}

int ckpt_read_lattice(FILE *f, lbm_lattice *l, int64_t *counter) {
    LatHeader hd{};
    if (fread(&hd, sizeof(hd), 1, f) != 1) return fail("checkpoint file is truncated");
    if (memcmp(hd.magic, kLatMagic, 8)) return fail("not a lattice checkpoint (bad magic)");
    if (hd.storage != l->storage || hd.nx != l->nx || hd.ny != l->ny || hd.nz != l->nz)
        return fail("checkpoint lattice size or storage type does not match");
    const size_t eb = storage_bytes(l->storage), pb = (size_t)l->n * eb;
    Staging sg;
    if (sg.init(std::min(kChunk, std::max(pb, (size_t)l->n)))) return -1;
    Fnv h;
    if (read_region(f, l->flags, (size_t)l->n, sg, h)) return -1;
    for (int i = 0; i < 19; i++)
        if (read_region(f, (unsigned char *)l->dd + (size_t)i * l->pstride * eb, pb, sg, h)) return -1;
    uint64_t want = 0;
    if (fread(&want, sizeof(want), 1, f) != 1) return fail("checkpoint file is truncated");
    if (want != h.h) return fail("checkpoint hash mismatch (corrupt file)");
    if (counter) *counter = hd.counter;
    return 0;
}

}  // namespace lbm_rt

extern "C" {

int lbm_cu_checkpoint_save(lbm_lattice *lat, const char *path, int64_t counter, void *stream) {
    if (!lat || !path) return fail("NULL argument");
    if (counter < 0) return fail("negative step counter");
    CU(cudaStreamSynchronize(S(stream)));
    File fh;
    fh.f = fopen(path, "wb");
    if (!fh.f) return fail(std::string("cannot open ") + path + " for writing");
    if (ckpt_write_lattice(fh.f, lat, counter)) return -1;
    if (fflush(fh.f)) return fail("checkpoint write failed");
    return 0;
}

int lbm_cu_checkpoint_load(lbm_lattice *lat, const char *path, int64_t *counter, void *stream) {
    if (!lat || !path) return fail("NULL argument");
    CU(cudaStreamSynchronize(S(stream)));
    File fh;
    fh.f = fopen(path, "rb");
    if (!fh.f) return fail(std::string("cannot open ") + path);
    return ckpt_read_lattice(fh.f, lat, counter);
}

}  // extern "C"
