// A small reader of the HDF5 files StePS writes its Ewald lookup tables to
// (save_t3_ewald_lookup_table / save_s1r2_ewald_lookup_table,
// StePS/src/inputoutput.cc:1792, :2102): the file layout the HDF5 library
// writes with default properties -- superblock version 0 or 1, version 1
// object headers, groups indexed by a symbol table (version 1 B-tree, symbol
// table nodes, local heap), datasets of IEEE floating point or integer
// elements stored contiguously (or compact). Anything else (chunked or
// filtered storage, newer object headers) is reported as unsupported.
//
// With it the library loads a table file written by the reference's driver
// unchanged, so the GPU and the reference's CPU path use the same table
// values without an HDF5 installation (steps_gpu_load_table_*_hdf5).
#include <stdint.h>
#include <stdio.h>
#include <string.h>

#include <string>
#include <vector>

#include "common.cuh"
#include "context.cuh"

namespace steps {

namespace {

struct H5File {
    std::vector<uint8_t> b;
    int so = 8, sl = 8;  // sizes of offsets and lengths
    uint64_t base = 0;   // base address

    // [at, at + n) lies in the file (no wrap-around for corrupt addresses)
    bool has(uint64_t at, uint64_t n) const { return at <= b.size() && n <= b.size() - at; }
    uint64_t u(uint64_t at, int n) const
    {
        if (!has(at, (uint64_t)n)) fail(STEPS_E_ARG, "hdf5: truncated file");
        uint64_t v = 0;
        for (int k = n - 1; k >= 0; k--) v = (v << 8) | b[at + k];
        return v;
    }
    // the 4-byte signature at `at` (bounds-checked)
    bool magic(uint64_t at, const char *sig) const { return has(at, 4) && memcmp(&b[at], sig, 4) == 0; }
    uint64_t off(uint64_t at) const { return u(at, so); }
    uint64_t len(uint64_t at) const { return u(at, sl); }
    uint64_t addr(uint64_t a) const { return a + base; }
    bool undef(uint64_t a) const { return so == 8 ? a == ~0ull : a == 0xffffffffull; }
};

struct Message {
    int type;
    uint64_t at;  // start of the message data
    uint64_t size;
};

// Messages of a version 1 object header, continuation blocks followed.
std::vector<Message> object_messages(const H5File &f, uint64_t oh)
{
    const uint64_t at = f.addr(oh);
    if (f.u(at, 1) != 1) fail(STEPS_E_ARG, "hdf5: only version 1 object headers are supported");
    const int nmsg = (int)f.u(at + 2, 2);
    std::vector<Message> out;
    std::vector<std::pair<uint64_t, uint64_t>> blocks{{at + 16, f.u(at + 8, 4)}};
    for (size_t bi = 0; bi < blocks.size() && (int)out.size() < nmsg; bi++) {
        uint64_t p = blocks[bi].first;
        const uint64_t end = p + blocks[bi].second;
        while (p + 8 <= end && (int)out.size() < nmsg) {
            const int type = (int)f.u(p, 2);
            const uint64_t size = f.u(p + 2, 2);
            if (p + 8 + size > end) fail(STEPS_E_ARG, "hdf5: object header message overruns its block");
            if (type == 0x10)  // continuation: offset, length
                blocks.emplace_back(f.addr(f.off(p + 8)), f.len(p + 8 + f.so));
            out.push_back({type, p + 8, size});
            p += 8 + size;
        }
    }
    return out;
}

std::string heap_name(const H5File &f, uint64_t heap, uint64_t offset)
{
    const uint64_t h = f.addr(heap);
    if (!f.magic(h, "HEAP")) fail(STEPS_E_ARG, "hdf5: bad local heap");
    const uint64_t data = f.addr(f.off(h + 8 + 2 * f.sl));
    std::string s;
    for (uint64_t p = data + offset; p < f.b.size() && f.b[p]; p++) s.push_back((char)f.b[p]);
    return s;
}

// Object header address of `name` in the group whose symbol table is
// (btree, heap): a walk of the version 1 group B-tree down to its symbol
// table nodes.
bool group_lookup(const H5File &f, uint64_t btree, uint64_t heap, const std::string &name, uint64_t &oh, int depth = 0)
{
    if (depth > 64) fail(STEPS_E_ARG, "hdf5: group B-tree too deep");
    const uint64_t t = f.addr(btree);
    if (!f.magic(t, "TREE") || f.u(t + 4, 1) != 0) fail(STEPS_E_ARG, "hdf5: bad group B-tree node");
    const int level = (int)f.u(t + 5, 1);
    const int used = (int)f.u(t + 6, 2);
    uint64_t p = t + 8 + 2 * f.so;  // key 0, child 0, key 1, child 1, ..., key `used`
    for (int k = 0; k < used; k++) {
        const uint64_t child = f.off(p + f.sl);
        p += f.sl + f.so;
        if (level > 0) {
            if (group_lookup(f, child, heap, name, oh, depth + 1)) return true;
            continue;
        }
        const uint64_t s = f.addr(child);
        if (!f.magic(s, "SNOD")) fail(STEPS_E_ARG, "hdf5: bad symbol table node");
        const int nsym = (int)f.u(s + 6, 2);
        const uint64_t entry = 2 * (uint64_t)f.so + 24;  // name offset, header address, cache type + pad, scratch
        for (int e = 0; e < nsym; e++) {
            const uint64_t q = s + 8 + e * entry;
            if (heap_name(f, heap, f.off(q)) == name) {
                oh = f.off(q + f.so);
                return true;
            }
        }
    }
    return false;
}

// Object header address of an absolute path "/a/b/c".
uint64_t resolve(const H5File &f, uint64_t root_oh, const std::string &path)
{
    uint64_t oh = root_oh;
    size_t pos = 0;
    while (pos < path.size()) {
        while (pos < path.size() && path[pos] == '/') pos++;
        if (pos >= path.size()) break;
        const size_t end = path.find('/', pos);
        const std::string part = path.substr(pos, end == std::string::npos ? std::string::npos : end - pos);
        pos = end == std::string::npos ? path.size() : end;
        uint64_t btree = 0, heap = 0;
        bool found = false;
        for (const Message &m : object_messages(f, oh))
            if (m.type == 0x11) {  // symbol table message: B-tree and heap addresses
                btree = f.off(m.at);
                heap = f.off(m.at + f.so);
                found = true;
            }
        if (!found) fail(STEPS_E_ARG, "hdf5: '" + part + "' is looked up in an object that is not a symbol-table group");
        if (!group_lookup(f, btree, heap, part, oh)) fail(STEPS_E_ARG, "hdf5: no object '" + part + "' in " + path);
    }
    return oh;
}

struct Dataset {
    std::vector<uint64_t> dims;
    int cls = -1;        // 0 fixed point, 1 floating point
    int size = 0;        // bytes per element
    bool is_signed = false;
    uint64_t data = 0;   // file offset of the raw data
    uint64_t bytes = 0;  // its size
};

Dataset read_dataset_header(const H5File &f, uint64_t oh)
{
    Dataset d;
    bool have_space = false, have_type = false, have_layout = false;
    for (const Message &m : object_messages(f, oh)) {
        const uint64_t a = m.at;
        if (m.type == 0x01) {  // dataspace
            const int ver = (int)f.u(a, 1), rank = (int)f.u(a + 1, 1);
            const uint64_t dims_at = ver == 1 ? a + 8 : a + 4;
            if (ver != 1 && ver != 2) fail(STEPS_E_ARG, "hdf5: unsupported dataspace message version");
            d.dims.clear();
            for (int k = 0; k < rank; k++) d.dims.push_back(f.len(dims_at + (uint64_t)k * f.sl));
            have_space = true;
        } else if (m.type == 0x03) {  // datatype
            const int cv = (int)f.u(a, 1);
            d.cls = cv & 15;
            const int bits0 = (int)f.u(a + 1, 1);
            if (bits0 & 1) fail(STEPS_E_ARG, "hdf5: big-endian data is not supported");
            d.is_signed = d.cls == 0 && (bits0 & 8);
            d.size = (int)f.u(a + 4, 4);
            have_type = true;
        } else if (m.type == 0x08) {  // data layout
            const int ver = (int)f.u(a, 1);
            if (ver != 3) fail(STEPS_E_ARG, "hdf5: unsupported data layout message version");
            const int cls = (int)f.u(a + 1, 1);
            if (cls == 1) {  // contiguous
                const uint64_t adr = f.off(a + 2);
                d.bytes = f.len(a + 2 + f.so);
                if (f.undef(adr)) fail(STEPS_E_ARG, "hdf5: dataset has no storage allocated");
                d.data = f.addr(adr);
            } else if (cls == 0) {  // compact: the data sit in the message
                d.bytes = f.u(a + 2, 2);
                d.data = a + 4;
            } else {
                fail(STEPS_E_ARG, "hdf5: chunked datasets are not supported");
            }
            have_layout = true;
        } else if (m.type == 0x0b) {
            fail(STEPS_E_ARG, "hdf5: filtered (compressed) datasets are not supported");
        }
    }
    if (!have_space || !have_type || !have_layout) fail(STEPS_E_ARG, "hdf5: object is not a dataset");
    if (d.cls != 0 && d.cls != 1) fail(STEPS_E_ARG, "hdf5: only integer and floating-point datasets are supported");
    if (d.cls == 1 && d.size != 4 && d.size != 8) fail(STEPS_E_ARG, "hdf5: unsupported floating-point size");
    if (d.cls == 0 && d.size != 1 && d.size != 2 && d.size != 4 && d.size != 8)
        fail(STEPS_E_ARG, "hdf5: unsupported integer size");
    uint64_t count = 1;
    for (uint64_t v : d.dims) {
        if (v != 0 && count > f.b.size() / v) fail(STEPS_E_ARG, "hdf5: dataspace larger than the file");
        count *= v;
    }
    if (count * (uint64_t)d.size != d.bytes) fail(STEPS_E_ARG, "hdf5: storage size does not match the dataspace");
    if (!f.has(d.data, d.bytes)) fail(STEPS_E_ARG, "hdf5: truncated dataset");
    return d;
}

H5File open_file(const char *path)
{
    if (!path) fail(STEPS_E_ARG, "hdf5: path is NULL");
    FILE *fp = fopen(path, "rb");
    if (!fp) fail(STEPS_E_ARG, std::string("hdf5: cannot open ") + path);
    H5File f;
    fseek(fp, 0, SEEK_END);
    const long n = ftell(fp);
    fseek(fp, 0, SEEK_SET);
    f.b.resize(n > 0 ? (size_t)n : 0);
    const size_t got = n > 0 ? fread(f.b.data(), 1, (size_t)n, fp) : 0;
    fclose(fp);
    if ((long)got != n) fail(STEPS_E_ARG, std::string("hdf5: cannot read ") + path);
    static const uint8_t sig[8] = {0x89, 'H', 'D', 'F', '\r', '\n', 0x1a, '\n'};
    if (f.b.size() < 96 || memcmp(f.b.data(), sig, 8) != 0) fail(STEPS_E_ARG, "hdf5: not an HDF5 file");
    return f;
}

// Root group object header address (superblock versions 0 and 1).
uint64_t superblock(H5File &f)
{
    const int ver = (int)f.b[8];
    if (ver != 0 && ver != 1) fail(STEPS_E_ARG, "hdf5: only superblock versions 0 and 1 are supported");
    f.so = f.b[13];
    f.sl = f.b[14];
    if ((f.so != 4 && f.so != 8) || (f.sl != 4 && f.sl != 8)) fail(STEPS_E_ARG, "hdf5: unsupported address size");
    const uint64_t p = 24 + (ver == 1 ? 4 : 0);  // group leaf / internal K, consistency flags (+ v1 indexed K)
    f.base = f.off(p);
    const uint64_t root_entry = p + 4 * (uint64_t)f.so;  // after base, free-space, EOF, driver addresses
    return f.off(root_entry + f.so);                      // link name offset, then object header address
}

// Reads dataset `name` as doubles (integers and floats converted).
std::vector<double> read_f64(const char *path, const char *name, std::vector<uint64_t> &dims)
{
    H5File f = open_file(path);
    const uint64_t root = superblock(f);
    const Dataset d = read_dataset_header(f, resolve(f, root, name ? name : ""));
    dims = d.dims;
    const uint64_t count = d.bytes / d.size;
    std::vector<double> out(count);
    const uint8_t *src = f.b.data() + d.data;
    for (uint64_t i = 0; i < count; i++) {
        const uint8_t *e = src + i * d.size;
        if (d.cls == 1 && d.size == 8) {
            double v;
            memcpy(&v, e, 8);
            out[i] = v;
        } else if (d.cls == 1) {
            float v;
            memcpy(&v, e, 4);
            out[i] = v;
        } else {
            uint64_t v = 0;
            for (int k = d.size - 1; k >= 0; k--) v = (v << 8) | e[k];
            if (d.is_signed && d.size < 8 && (v >> (8 * d.size - 1)) & 1) v |= ~0ull << (8 * d.size);
            out[i] = d.is_signed ? (double)(int64_t)v : (double)v;
        }
    }
    return out;
}

}  // namespace

}  // namespace steps

using namespace steps;

extern "C" {

int steps_h5_read_f64(const char *path, const char *dataset, double *out, long long capacity, long long *count,
                      int *rank, long long *dims)
{
    struct A {
        const char *path, *dataset;
        double *out;
        long long capacity, *count;
        int *rank;
        long long *dims;
    } a{path, dataset, out, capacity, count, rank, dims};
    return run_guarded(
        [](void *vp) {
            A &a = *static_cast<A *>(vp);
            std::vector<uint64_t> d;
            std::vector<double> v = read_f64(a.path, a.dataset, d);
            if (a.rank) *a.rank = (int)d.size();
            if (a.dims)
                for (size_t k = 0; k < d.size() && k < 32; k++) a.dims[k] = (long long)d[k];
            if (a.count) *a.count = (long long)v.size();
            if (a.out) {
                if ((long long)v.size() > a.capacity) fail(STEPS_E_ARG, "hdf5: dataset larger than the buffer");
                memcpy(a.out, v.data(), v.size() * sizeof(double));
            }
        },
        &a);
}

int steps_gpu_load_table_t3_hdf5(const char *path, int *ngrid_out)
{
    struct A {
        const char *path;
        int *ngrid;
    } a{path, ngrid_out};
    return run_guarded(
        [](void *vp) {
            A &a = *static_cast<A *>(vp);
            std::vector<uint64_t> d;
            std::vector<double> t = read_f64(a.path, "/t3_ewald/T3_EWALD_FORCE_TABLE", d);
            if (d.size() != 4 || d[3] != 3 || d[0] != d[1] || d[1] != d[2] || d[0] < 2 || d[0] > 1024)
                fail(STEPS_E_TABLE, "hdf5: T3_EWALD_FORCE_TABLE is not (Ng, Ng, Ng, 3)");
            const int ng = (int)d[0];
            int rc = steps_gpu_set_table_t3(ng, t.data());
            if (rc != STEPS_OK) fail(rc, steps_gpu_error_string());
            if (a.ngrid) *a.ngrid = ng;
        },
        &a);
}

int steps_gpu_load_table_s1r2_hdf5(const char *path, int *nrho_out, int *nz_out)
{
    struct A {
        const char *path;
        int *nrho, *nz;
    } a{path, nrho_out, nz_out};
    return run_guarded(
        [](void *vp) {
            A &a = *static_cast<A *>(vp);
            std::vector<uint64_t> d;
            std::vector<double> t = read_f64(a.path, "/s1r2_ewald/S1R2_EWALD_FORCE_TABLE", d);
            if (d.size() != 3 || d[2] != 2 || d[0] < 1 || d[1] < 1 || d[0] * d[1] > (1ull << 28))
                fail(STEPS_E_TABLE, "hdf5: S1R2_EWALD_FORCE_TABLE is not (Nrho, Nz, 2)");
            int rc = steps_gpu_set_table_s1r2((int)d[0], (int)d[1], t.data());
            if (rc != STEPS_OK) fail(rc, steps_gpu_error_string());
            if (a.nrho) *a.nrho = (int)d[0];
            if (a.nz) *a.nz = (int)d[1];
        },
        &a);
}

}  // extern "C"
