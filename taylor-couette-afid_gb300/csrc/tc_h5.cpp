// tc_h5.cpp -- the HDF5 files of the reference's restart path, without
// libhdf5: continua_q{t,r,z}.h5 (dataset "var", the interior of one velocity
// field), continua_master.h5 (grid and time scalars) and cordin_info.h5
// (coordinates), as WriteFlowField.F90:17-47, ReadFlowField.F90:31-149 and
// WriteGridInfo.F90:22-33 read and write them through HdfRoutines.F90.
//
// The subset of the HDF5 file format written and read here is the one the
// HDF5 1.8 library produces with its default properties:
//   superblock version 0 (or 1 on reading), 8-byte offsets and lengths;
//   groups as symbol tables: a version-1 B-tree of group nodes over symbol
//   table nodes, names in a local heap;
//   version-1 object headers (with continuation blocks on reading);
//   datasets with a simple dataspace (message versions 1 and 2), a fixed-
//   point or IEEE floating-point little-endian datatype, and contiguous (or,
//   on reading, compact) storage.
// Writing uses one symbol table node for all the names of a file (its group
// leaf K is raised to fit them), contiguous storage and no fill value.
//
// Layout of the reference's arrays: Fortran q(1:nr, 1:nzm, 1:nthm) is the
// HDF5 dataspace [nthm][nzm][nr] (the Fortran API lists dimensions in
// reverse), r fastest.

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/tc_capi.h"

namespace tcgb {
void set_last_error(const std::string& msg);
void set_handle_error(tc_handle* h, const std::string& msg);
}

namespace {

constexpr uint64_t kUndef = ~0ull;

// ---------------------------------------------------------------------------
// writing

struct WDataset {
    std::string name;
    bool is_int;                 // int32 (H5T_NATIVE_INTEGER) or float64
    std::vector<uint64_t> dims;
    std::vector<uint8_t> bytes;  // little-endian element data
};

struct Buf {
    std::vector<uint8_t> b;
    void u8(uint8_t v) { b.push_back(v); }
    void u16(uint16_t v) { for (int i = 0; i < 2; ++i) b.push_back((uint8_t)(v >> (8 * i))); }
    void u32(uint32_t v) { for (int i = 0; i < 4; ++i) b.push_back((uint8_t)(v >> (8 * i))); }
    void u64(uint64_t v) { for (int i = 0; i < 8; ++i) b.push_back((uint8_t)(v >> (8 * i))); }
    void zeros(size_t n) { b.insert(b.end(), n, 0); }
    void pad8() { while (b.size() % 8) b.push_back(0); }
    size_t size() const { return b.size(); }
};

// One object-header message: type, payload padded to 8 bytes.
void message(Buf& o, uint16_t type, uint8_t flags, const Buf& payload) {
    Buf p = payload;
    p.pad8();
    o.u16(type);
    o.u16((uint16_t)p.size());
    o.u8(flags);
    o.zeros(3);
    o.b.insert(o.b.end(), p.b.begin(), p.b.end());
}

// Version-1 object header holding `msgs` (already encoded messages).
void object_header(Buf& out, const Buf& msgs, int nmsgs) {
    out.u8(1);                       // version
    out.u8(0);
    out.u16((uint16_t)nmsgs);
    out.u32(1);                      // reference count
    out.u32((uint32_t)msgs.size());  // header data size
    out.zeros(4);                    // align the messages to 8 bytes
    out.b.insert(out.b.end(), msgs.b.begin(), msgs.b.end());
}

Buf dataset_messages(const WDataset& d, uint64_t data_addr, int* nmsgs) {
    Buf m;
    {   // dataspace, version 1
        Buf p;
        p.u8(1);
        p.u8((uint8_t)d.dims.size());
        p.u8(0);                     // no maximum dimensions
        p.zeros(5);
        for (uint64_t x : d.dims) p.u64(x);
        message(m, 0x0001, 0, p);
    }
    {   // datatype, version 1
        Buf p;
        if (d.is_int) {
            p.u8(0x10);              // class 0: fixed point
            p.u8(0x08); p.u8(0); p.u8(0);   // little endian, signed
            p.u32(4);
            p.u16(0); p.u16(32);     // bit offset, precision
        } else {
            p.u8(0x11);              // class 1: floating point
            p.u8(0x20); p.u8(63); p.u8(0);  // little endian, implied msb, sign bit 63
            p.u32(8);
            p.u16(0); p.u16(64);     // bit offset, precision
            p.u8(52); p.u8(11);      // exponent location, size
            p.u8(0); p.u8(52);       // mantissa location, size
            p.u32(1023);             // exponent bias
        }
        message(m, 0x0003, 1, p);
    }
    {   // fill value, version 2: allocation late, written if set, undefined
        Buf p;
        p.u8(2); p.u8(2); p.u8(2); p.u8(0);
        message(m, 0x0005, 1, p);
    }
    {   // data layout, version 3, contiguous
        Buf p;
        p.u8(3);
        p.u8(1);
        p.u64(data_addr);
        p.u64((uint64_t)d.bytes.size());
        message(m, 0x0008, 0, p);
    }
    *nmsgs = 4;
    return m;
}

bool write_file(const std::string& path, std::vector<WDataset> ds, std::string& err) {
    std::sort(ds.begin(), ds.end(), [](const WDataset& a, const WDataset& b) { return a.name < b.name; });
    const int n = (int)ds.size();
    const int leafK = std::max(4, (n + 1) / 2);      // a symbol table node holds 2K entries
    const int nodeK = 16;                            // group B-tree node: 2K children
    // local heap data: "" at 0, then the names, each padded to 8 bytes
    Buf heap;
    heap.zeros(8);
    std::vector<uint64_t> name_off(n);
    for (int i = 0; i < n; ++i) {
        name_off[i] = heap.size();
        heap.b.insert(heap.b.end(), ds[i].name.begin(), ds[i].name.end());
        heap.u8(0);
        heap.pad8();
    }
    // addresses
    const uint64_t a_root = 96;                      // after the 96-byte superblock
    const uint64_t root_size = 16 + 8 + 16;
    const uint64_t a_heap = a_root + root_size;
    const uint64_t a_heapdata = a_heap + 32;
    const uint64_t a_btree = a_heapdata + heap.size();
    const uint64_t btree_size = 24 + (2 * nodeK + 1) * 8 + 2 * nodeK * 8;
    const uint64_t a_snod = a_btree + btree_size;
    const uint64_t snod_size = 8 + 2 * (uint64_t)leafK * 40;
    uint64_t a = a_snod + snod_size;
    std::vector<uint64_t> a_oh(n), a_data(n);
    std::vector<Buf> ohs(n);
    for (int i = 0; i < n; ++i) {   // header sizes do not depend on the data address
        int nm = 0;
        Buf msgs = dataset_messages(ds[i], 0, &nm);
        a_oh[i] = a;
        a += 16 + msgs.size();
    }
    for (int i = 0; i < n; ++i) {
        a_data[i] = a;
        a += ds[i].bytes.size();
        a = (a + 7) & ~7ull;
    }
    const uint64_t eof = a;
    for (int i = 0; i < n; ++i) {
        int nm = 0;
        Buf msgs = dataset_messages(ds[i], a_data[i], &nm);
        object_header(ohs[i], msgs, nm);
    }

    Buf f;
    // superblock version 0
    const uint8_t sig[8] = {0x89, 'H', 'D', 'F', '\r', '\n', 0x1a, '\n'};
    f.b.insert(f.b.end(), sig, sig + 8);
    f.u8(0); f.u8(0); f.u8(0); f.u8(0);   // superblock, free space, root entry versions; reserved
    f.u8(0); f.u8(8); f.u8(8); f.u8(0);   // shared header version, offset size, length size, reserved
    f.u16((uint16_t)leafK);
    f.u16((uint16_t)nodeK);
    f.u32(0);                            // consistency flags
    f.u64(0);                            // base address
    f.u64(kUndef);                       // free-space info
    f.u64(eof);
    f.u64(kUndef);                       // driver information block
    // root group symbol table entry, scratch pad caching the group's tables
    f.u64(0);
    f.u64(a_root);
    f.u32(1);
    f.u32(0);
    f.u64(a_btree);
    f.u64(a_heap);
    // root group object header: one symbol table message
    {
        Buf p;
        p.u64(a_btree);
        p.u64(a_heap);
        Buf msgs;
        message(msgs, 0x0011, 0, p);
        object_header(f, msgs, 1);
    }
    // local heap
    f.b.insert(f.b.end(), {'H', 'E', 'A', 'P'});
    f.u8(0); f.zeros(3);
    f.u64(heap.size());
    f.u64(kUndef);                       // no free block
    f.u64(a_heapdata);
    f.b.insert(f.b.end(), heap.b.begin(), heap.b.end());
    // group B-tree: one leaf node with one child, the symbol table node
    f.b.insert(f.b.end(), {'T', 'R', 'E', 'E'});
    f.u8(0);                             // group node
    f.u8(0);                             // level 0
    f.u16(n > 0 ? 1 : 0);
    f.u64(kUndef);
    f.u64(kUndef);
    f.u64(0);                            // key 0: the empty name
    f.u64(a_snod);                       // child 0
    f.u64(n > 0 ? name_off[n - 1] : 0);  // key 1: the last name in child 0
    f.zeros((size_t)(btree_size - 24 - 3 * 8));
    // symbol table node
    f.b.insert(f.b.end(), {'S', 'N', 'O', 'D'});
    f.u8(1); f.u8(0);
    f.u16((uint16_t)n);
    for (int i = 0; i < n; ++i) {
        f.u64(name_off[i]);
        f.u64(a_oh[i]);
        f.u32(0); f.u32(0);
        f.zeros(16);
    }
    f.zeros((size_t)(2 * leafK - n) * 40);
    for (int i = 0; i < n; ++i) {
        if (f.size() != a_oh[i]) { err = "internal layout error"; return false; }
        f.b.insert(f.b.end(), ohs[i].b.begin(), ohs[i].b.end());
    }
    for (int i = 0; i < n; ++i) {
        while (f.size() < a_data[i]) f.u8(0);
        f.b.insert(f.b.end(), ds[i].bytes.begin(), ds[i].bytes.end());
    }
    while (f.size() < eof) f.u8(0);
    FILE* fp = std::fopen(path.c_str(), "wb");
    if (!fp) { err = "cannot create " + path; return false; }
    const size_t w = std::fwrite(f.b.data(), 1, f.size(), fp);
    const bool ok = std::fclose(fp) == 0 && w == f.size();
    if (!ok) err = "write failed: " + path;
    return ok;
}

WDataset f64_dataset(const std::string& name, std::vector<uint64_t> dims, const double* v) {
    WDataset d{name, false, dims, {}};
    uint64_t n = 1;
    for (uint64_t x : dims) n *= x;
    d.bytes.resize(n * 8);
    for (uint64_t i = 0; i < n; ++i) {
        uint64_t u;
        std::memcpy(&u, v + i, 8);
        for (int b = 0; b < 8; ++b) d.bytes[i * 8 + b] = (uint8_t)(u >> (8 * b));
    }
    return d;
}

WDataset i32_dataset(const std::string& name, int32_t v) {
    WDataset d{name, true, {1}, {}};
    const uint32_t u = (uint32_t)v;
    for (int b = 0; b < 4; ++b) d.bytes.push_back((uint8_t)(u >> (8 * b)));
    return d;
}

// ---------------------------------------------------------------------------
// reading

struct Reader {
    std::vector<uint8_t> f;
    std::string err;
    int leafK = 4, nodeK = 16;

    bool load(const std::string& path) {
        FILE* fp = std::fopen(path.c_str(), "rb");
        if (!fp) { err = "cannot open " + path; return false; }
        std::fseek(fp, 0, SEEK_END);
        long sz = std::ftell(fp);
        std::fseek(fp, 0, SEEK_SET);
        if (sz < 0) { std::fclose(fp); err = "cannot size " + path; return false; }
        f.resize((size_t)sz);
        size_t r = sz > 0 ? std::fread(f.data(), 1, (size_t)sz, fp) : 0;
        std::fclose(fp);
        if (r != (size_t)sz) { err = "short read: " + path; return false; }
        return true;
    }
    bool have(uint64_t at, uint64_t n) {
        if (at > f.size() || n > f.size() - at) { err = "truncated or corrupt file"; return false; }
        return true;
    }
    uint64_t le(uint64_t at, int n) const {
        uint64_t v = 0;
        for (int i = 0; i < n; ++i) v |= (uint64_t)f[at + i] << (8 * i);
        return v;
    }

    // superblock -> root group (B-tree, heap) addresses
    bool root(uint64_t* btree, uint64_t* heap) {
        static const uint8_t sig[8] = {0x89, 'H', 'D', 'F', '\r', '\n', 0x1a, '\n'};
        if (!have(0, 8) || std::memcmp(f.data(), sig, 8) != 0) { err = "not an HDF5 file (no signature at 0)"; return false; }
        if (!have(8, 16)) return false;
        const int ver = f[8];
        if (ver > 1) { err = "superblock version " + std::to_string(ver) + " is not supported"; return false; }
        if (f[13] != 8 || f[14] != 8) { err = "only 8-byte offsets and lengths are supported"; return false; }
        leafK = (int)le(16, 2);
        nodeK = (int)le(18, 2);
        uint64_t p = 24;
        if (ver == 1) p += 4;
        p += 32;                        // base, free space, eof, driver
        if (!have(p, 40)) return false;
        const uint64_t oh = le(p + 8, 8);
        return group_tables(oh, btree, heap);
    }

    // Walk the messages of a version-1 object header (with continuations).
    template <typename F>
    bool messages(uint64_t oh, F fn) {
        if (!have(oh, 16)) return false;
        if (f[oh] != 1) {
            err = (f[oh] == 'O') ? "version-2 object headers are not supported" : "bad object header";
            return false;
        }
        const int nmsg = (int)le(oh + 2, 2);
        std::vector<std::pair<uint64_t, uint64_t>> blocks{{oh + 16, le(oh + 8, 4)}};
        int seen = 0;
        for (size_t bi = 0; bi < blocks.size() && seen < nmsg; ++bi) {
            uint64_t p = blocks[bi].first, end = p + blocks[bi].second;
            if (!have(p, blocks[bi].second)) return false;
            while (p + 8 <= end && seen < nmsg) {
                const int type = (int)le(p, 2), size = (int)le(p + 2, 2);
                const uint64_t data = p + 8;
                if (!have(data, (uint64_t)size)) return false;
                ++seen;
                if (type == 0x0010) {
                    blocks.push_back({le(data, 8), le(data + 8, 8)});
                } else if (!fn(type, data, size)) {
                    return false;
                }
                p = data + size;
            }
        }
        return true;
    }

    bool group_tables(uint64_t oh, uint64_t* btree, uint64_t* heap) {
        bool found = false;
        if (!messages(oh, [&](int type, uint64_t d, int) {
                if (type == 0x0011) {
                    *btree = le(d, 8);
                    *heap = le(d + 8, 8);
                    found = true;
                }
                return true;
            }))
            return false;
        if (!found) { err = "the root group has no symbol table (new-style groups are not supported)"; return false; }
        return true;
    }

    // name -> object header address through the group B-tree
    bool lookup(uint64_t btree, uint64_t heap, const std::string& name, uint64_t* oh) {
        if (!have(heap, 32) || std::memcmp(&f[heap], "HEAP", 4) != 0) { err = "bad local heap"; return false; }
        const uint64_t hdata = le(heap + 24, 8), hsize = le(heap + 8, 8);
        if (!have(hdata, hsize)) return false;
        return search(btree, hdata, hsize, name, oh, 0);
    }

    bool search(uint64_t node, uint64_t hdata, uint64_t hsize, const std::string& name, uint64_t* oh, int depth) {
        if (depth > 32) { err = "B-tree too deep"; return false; }
        if (!have(node, 24)) return false;
        if (std::memcmp(&f[node], "TREE", 4) == 0) {
            if (f[node + 4] != 0) { err = "not a group B-tree"; return false; }
            const int n = (int)le(node + 6, 2);
            if (!have(node + 24, (uint64_t)(2 * n + 1) * 8)) return false;
            for (int c = 0; c < n; ++c) {
                const uint64_t child = le(node + 24 + 8 + 16 * (uint64_t)c, 8);
                if (search(child, hdata, hsize, name, oh, depth + 1)) return true;
                if (!err.empty()) return false;
            }
            return false;
        }
        if (std::memcmp(&f[node], "SNOD", 4) == 0) {
            const int n = (int)le(node + 6, 2);
            if (!have(node + 8, (uint64_t)n * 40)) return false;
            for (int e = 0; e < n; ++e) {
                const uint64_t ent = node + 8 + 40 * (uint64_t)e;
                const uint64_t off = le(ent, 8);
                if (off >= hsize) { err = "bad name offset"; return false; }
                const char* s = (const char*)&f[hdata + off];
                const size_t len = strnlen(s, (size_t)(hsize - off));
                if (name == std::string(s, len)) {
                    *oh = le(ent + 8, 8);
                    return true;
                }
            }
            return false;
        }
        err = "bad B-tree node";
        return false;
    }

    // a dataset as doubles
    bool dataset(uint64_t oh, std::vector<double>& out, std::vector<uint64_t>& dims) {
        int cls = -1, size = 0, order = 0;
        bool sgn = true;
        bool have_space = false, have_layout = false;
        uint64_t addr = kUndef, bytes = 0, compact = 0;
        bool is_compact = false;
        if (!messages(oh, [&](int type, uint64_t d, int) {
                if (type == 0x0001) {
                    const int ver = f[d], rank = f[d + 1];
                    const uint64_t p = d + (ver == 1 ? 8 : 4);
                    dims.clear();
                    for (int r = 0; r < rank; ++r) dims.push_back(le(p + 8 * (uint64_t)r, 8));
                    have_space = true;
                } else if (type == 0x0003) {
                    cls = f[d] & 0x0f;
                    order = f[d + 1] & 1;
                    sgn = (f[d + 1] & 0x08) != 0;
                    size = (int)le(d + 4, 4);
                } else if (type == 0x0008) {
                    const int ver = f[d];
                    if (ver != 3) { err = "data layout message version " + std::to_string(ver) + " is not supported"; return false; }
                    const int lc = f[d + 1];
                    if (lc == 1) {
                        addr = le(d + 2, 8);
                        bytes = le(d + 10, 8);
                    } else if (lc == 0) {
                        bytes = le(d + 2, 2);
                        compact = d + 4;
                        is_compact = true;
                    } else {
                        err = "chunked storage is not supported";
                        return false;
                    }
                    have_layout = true;
                } else if (type == 0x000B) {
                    err = "filtered (compressed) datasets are not supported";
                    return false;
                }
                return true;
            }))
            return false;
        if (!have_space || !have_layout || cls < 0) { err = "incomplete dataset header"; return false; }
        if (order != 0) { err = "big-endian data is not supported"; return false; }
        uint64_t n = 1;
        for (uint64_t x : dims) n *= x;
        if (!((cls == 1 && (size == 8 || size == 4)) || (cls == 0 && (size == 4 || size == 8)))) {
            err = "unsupported datatype (class " + std::to_string(cls) + ", size " + std::to_string(size) + ")";
            return false;
        }
        if (bytes < n * (uint64_t)size) { err = "dataset storage smaller than its dataspace"; return false; }
        const uint64_t src = is_compact ? compact : addr;
        if (!is_compact && addr == kUndef) { err = "dataset has no storage allocated"; return false; }
        if (!have(src, n * (uint64_t)size)) return false;
        out.resize(n);
        for (uint64_t i = 0; i < n; ++i) {
            const uint64_t u = le(src + i * size, size);
            if (cls == 1 && size == 8) { double v; std::memcpy(&v, &u, 8); out[i] = v; }
            else if (cls == 1) { uint32_t w = (uint32_t)u; float v; std::memcpy(&v, &w, 4); out[i] = v; }
            else if (size == 4) out[i] = sgn ? (double)(int32_t)(uint32_t)u : (double)(uint32_t)u;
            else out[i] = sgn ? (double)(int64_t)u : (double)u;
        }
        return true;
    }
};

bool read_named(const std::string& path, const std::string& name, std::vector<double>& out,
                std::vector<uint64_t>& dims, std::string& err) {
    Reader r;
    uint64_t bt = 0, hp = 0, oh = 0;
    if (!r.load(path) || !r.root(&bt, &hp)) { err = r.err; return false; }
    if (!r.lookup(bt, hp, name, &oh)) {
        err = r.err.empty() ? "no dataset '" + name + "' in " + path : r.err;
        return false;
    }
    if (!r.dataset(oh, out, dims)) { err = r.err; return false; }
    return true;
}

int fail(int code, const std::string& msg) {
    tcgb::set_last_error(msg);
    return code;
}

int hfail(tc_handle* h, int code, const std::string& msg) {
    tcgb::set_handle_error(h, msg);
    return code;
}

std::string join(const char* dir, const char* file) {
    std::string d = dir ? dir : ".";
    if (d.empty()) d = ".";
    if (d.back() != '/') d += '/';
    return d + file;
}

}  // namespace

// ---- exported (declared extern "C" in tc_capi.h) ---------------------------

int tc_h5_write_dataset(const char* path, const char* name, int rank, const long long* dims, const double* data) {
    if (!path || !name || !dims || !data || rank < 1 || rank > 8) return fail(2000, "tc_h5_write_dataset: bad argument");
    std::vector<uint64_t> d;
    for (int r = 0; r < rank; ++r) {
        if (dims[r] < 1) return fail(2000, "tc_h5_write_dataset: dimensions must be positive");
        d.push_back((uint64_t)dims[r]);
    }
    std::string err;
    if (!write_file(path, {f64_dataset(name, d, data)}, err)) return fail(2021, err);
    return 0;
}

int tc_h5_read_dataset(const char* path, const char* name, double* out, long long cap, int* rank, long long* dims) {
    if (!path || !name) return fail(2000, "tc_h5_read_dataset: bad argument");
    std::vector<double> v;
    std::vector<uint64_t> d;
    std::string err;
    if (!read_named(path, name, v, d, err)) return fail(2022, err);
    if (rank) *rank = (int)d.size();
    if (dims) for (size_t r = 0; r < d.size() && r < 8; ++r) dims[r] = (long long)d[r];
    if (out) {
        if ((long long)v.size() > cap) return fail(2023, "tc_h5_read_dataset: output buffer too small");
        std::memcpy(out, v.data(), v.size() * sizeof(double));
    }
    return 0;
}

int tc_h5_write_continua(tc_handle* h, const char* dir, double time) {
    tc_bou b;
    if (!h || tc_get_bou(h, &b)) return hfail(h, 2000, "tc_h5_write_continua: null handle");
    const tc_bou* cfg = &b;
    const int nthm = cfg->nthm, nzm = cfg->nzm, nrm = cfg->nrm, nr = nrm + 1;
    const size_t halo = (size_t)(nthm + 2) * (nzm + 2) * nr;
    std::vector<double> q[3];
    for (auto& a : q) a.resize(halo);
    if (int r = tc_get_state(h, q[0].data(), q[1].data(), q[2].data(), nullptr)) return r;
    // interior q(1:nr, 1:nzm, 1:nthm) of q(1:nr, 0:nzm+1, 0:nthm+1)
    const char* files[3] = {"continua_qt.h5", "continua_qr.h5", "continua_qz.h5"};
    std::vector<double> in((size_t)nthm * nzm * nr);
    for (int c = 0; c < 3; ++c) {
        for (int i = 0; i < nthm; ++i)
            for (int j = 0; j < nzm; ++j)
                std::memcpy(&in[((size_t)i * nzm + j) * nr], &q[c][((size_t)(i + 1) * (nzm + 2) + (j + 1)) * nr],
                            sizeof(double) * nr);
        std::string err;
        if (!write_file(join(dir, files[c]), {f64_dataset("var", {(uint64_t)nthm, (uint64_t)nzm, (uint64_t)nr}, in.data())}, err))
            return hfail(h, 2021, err);
    }
    std::vector<WDataset> m;
    m.push_back(i32_dataset("nr", nr));
    m.push_back(i32_dataset("nth", nthm + 1));
    m.push_back(i32_dataset("nz", nzm + 1));
    m.push_back(f64_dataset("time", {1}, &time));
    m.push_back(f64_dataset("rint", {1}, &cfg->rint));
    m.push_back(f64_dataset("rext", {1}, &cfg->rext));
    m.push_back(i32_dataset("istr", cfg->istr));
    m.push_back(f64_dataset("str", {1}, &cfg->str));
    m.push_back(f64_dataset("alx3", {1}, &cfg->alx3));
    m.push_back(f64_dataset("lamb", {1}, &cfg->lamb));
    std::string err;
    if (!write_file(join(dir, "continua_master.h5"), m, err)) return hfail(h, 2021, err);
    return 0;
}

// ---- restart interpolation (interp.F90), for ReadFlowField's grid change ----

namespace {

// interp.F90:262-303 (gridnew): n points rc(1:n) and mid points rm(1:n),
// 1-based in out vectors of size n + 2 (index 0 and n + 1 are filled later).
// For istr = 0 it computes rc = rext x + rint, not (rext - rint) x + rint;
// kept, as the reference interpolates between grids built the same way.
bool gridnew(int n, double rint, double rext, int istr, double str, std::vector<double>& rc, std::vector<double>& rm) {
    rc.assign(n + 2, 0.0);
    rm.assign(n + 2, 0.0);
    if (istr == 0) {
        for (int i = 1; i <= n; ++i) {
            const double x3 = (double)(i - 1) / (double)(n - 1);
            rc[i] = rext * x3 + rint;
        }
    } else if (istr == 6) {
        const double pi = 2.0 * std::asin(1.0);
        const int nclip = (int)str;
        const int nrmo = n + nclip + nclip;
        std::vector<double> etazm(nrmo + 1), etaz(n + 1);
        for (int i = 1; i <= nrmo; ++i) etazm[i] = +std::cos(pi * ((double)i - 0.5) / (double)nrmo);
        for (int i = 1; i <= n; ++i) etaz[i] = etazm[i + nclip];
        const double delet = etaz[1] - etaz[n];
        for (int i = 1; i <= n; ++i) etaz[i] = etaz[i] / (0.5 * delet);
        rc[1] = rint;
        for (int i = 2; i <= n - 1; ++i) rc[i] = (rext - rint) * (1. - etaz[i]) * 0.5 + rint;
        rc[n] = rext;
    } else {
        return false;
    }
    for (int i = 1; i <= n - 1; ++i) rm[i] = (rc[i] + rc[i + 1]) * 0.5;
    rm[n] = 2 * rc[n] - rm[n - 1];
    return true;
}

// interp.F90:1-215 for one field: `old` holds q(1:nro, 1:nzom, 1:nthom)
// (r fastest); the result q(1:nr, 1:nzm, 1:nthm) goes to `out`.
// Reference behaviour kept: the field is placed at (tc, zm, rm) for intvar 1
// (qt), (tm, zc, rm) for 2 (qr) and (tm, zm, rc) for 3 (qz); the halos of the
// old field are linear extrapolations; the radial "upper" corner values are
// taken from the lower plane bifk (interp.F90:166-169), so the radial
// direction is not interpolated.
void interp_field(const std::vector<double>& old, int ntho, int nzo, int nro, int istro, double stro, int intvar,
                  const tc_bou& b, std::vector<double>& out) {
    const int nthom = ntho - 1, nzom = nzo - 1;
    const int nthm = b.nthm, nzm = b.nzm, nr = b.nrm + 1;
    const double pi = 2.0 * std::asin(1.0);
    const double thmax = 2.0 * pi / b.lamb;
    std::vector<double> tcold, tmold, zcold, zmold, rcold, rmold, tcnew, tmnew, zcnew, zmnew, rcnew, rmnew;
    gridnew(ntho, 0.0, thmax, 0, 1.0, tcold, tmold);
    gridnew(nzo, 0.0, b.alx3, 0, 1.0, zcold, zmold);
    gridnew(nro, b.rint, b.rext, istro, stro, rcold, rmold);
    auto ends = [](std::vector<double>& a, int n) {
        a[0] = 2 * a[1] - a[2];
        a[n + 1] = 2 * a[n] - a[n - 1];
    };
    ends(tcold, ntho); ends(tmold, ntho); ends(zcold, nzo); ends(zmold, nzo); ends(rcold, nro); ends(rmold, nro);
    gridnew(nthm + 1, 0.0, thmax, 0, 1.0, tcnew, tmnew);
    gridnew(nzm + 1, 0.0, b.alx3, 0, 1.0, zcnew, zmnew);
    gridnew(nr, b.rint, b.rext, b.istr, b.str, rcnew, rmnew);
    const std::vector<double>*xo, *yo, *zo, *xn, *yn, *zn;
    switch (intvar) {
        case 1: xo = &tcold; yo = &zmold; zo = &rmold; xn = &tcnew; yn = &zmnew; zn = &rmnew; break;
        case 2: xo = &tmold; yo = &zcold; zo = &rmold; xn = &tmnew; yn = &zcnew; zn = &rmnew; break;
        default: xo = &tmold; yo = &zmold; zo = &rcold; xn = &tmnew; yn = &zmnew; zn = &rcnew; break;
    }
    // arrold(0:nro+1, 0:nzom+1, 0:nthom+1); corners never set stay 0
    const size_t sk = 1, sj = (size_t)nro + 2, si = sj * (size_t)(nzom + 2);
    std::vector<double> a(si * (size_t)(nthom + 2), 0.0);
    auto A = [&](int k, int j, int i) -> double& { return a[(size_t)k * sk + (size_t)j * sj + (size_t)i * si]; };
    for (int i = 1; i <= nthom; ++i)
        for (int j = 1; j <= nzom; ++j)
            for (int k = 1; k <= nro; ++k) A(k, j, i) = old[(size_t)(k - 1) + (size_t)nro * ((size_t)(j - 1) + (size_t)nzom * (i - 1))];
    for (int i = 1; i <= nthom; ++i)                     // interp.F90:109-114
        for (int j = 1; j <= nzom; ++j) {
            A(0, j, i) = 2.0 * A(1, j, i) - A(2, j, i);
            A(nro + 1, j, i) = 2.0 * A(nro, j, i) - A(nro - 1, j, i);
        }
    for (int j = 1; j <= nzom; ++j)                      // interp.F90:116-121
        for (int k = 1; k <= nro; ++k) {
            A(k, j, 0) = 2.0 * A(k, j, 1) - A(k, j, 2);
            A(k, j, nthom + 1) = 2.0 * A(k, j, nthom) - A(k, j, nthom - 1);
        }
    for (int i = 1; i <= nthom; ++i)                     // interp.F90:123-128
        for (int k = 1; k <= nro; ++k) {
            A(k, 0, i) = 2.0 * A(k, 1, i) - A(k, 2, i);
            A(k, nzom + 1, i) = 2.0 * A(k, nzom, i) - A(k, nzom - 1, i);
        }
    auto bracket = [](const std::vector<double>& g, int n, double x, int& lo, int& hi) {
        lo = n - 1; hi = n;
        for (int l = 1; l <= n; ++l)
            if (g[l] >= x) { lo = l - 1; hi = l; return; }
    };
    out.assign((size_t)nr * nzm * nthm, 0.0);
    for (int i = 1; i <= nthm; ++i)
        for (int j = 1; j <= nzm; ++j)
            for (int k = 1; k <= nr; ++k) {
                const double bix = (*xn)[i], biy = (*yn)[j], biz = (*zn)[k];
                int bifi, bici, bifj, bicj, bifk, bick;
                bracket(*xo, ntho, bix, bifi, bici);
                bracket(*yo, nzo, biy, bifj, bicj);
                bracket(*zo, nro, biz, bifk, bick);
                const double bix1 = (*xo)[bifi], bix2 = (*xo)[bici];
                const double biy1 = (*yo)[bifj], biy2 = (*yo)[bicj];
                const double biz1 = (*zo)[bifk], biz2 = (*zo)[bick];
                const double sfcf = A(bifk, bicj, bifi), sfff = A(bifk, bifj, bifi);
                const double sccf = A(bifk, bicj, bici), scff = A(bifk, bifj, bici);
                const double sfcc = A(bifk, bicj, bifi), sffc = A(bifk, bifj, bifi);
                const double sccc = A(bifk, bicj, bici), scfc = A(bifk, bifj, bici);
                // interptrilin (interp.F90:218-258)
                const double dxdydz = 1.0 / ((bix2 - bix1) * (biy2 - biy1) * (biz2 - biz1));
                const double ans = (sfcf * (bix2 - bix) * (biy - biy1) * (biz2 - biz)
                                    + sfff * (bix2 - bix) * (biy2 - biy) * (biz2 - biz)
                                    + sccf * (bix - bix1) * (biy - biy1) * (biz2 - biz)
                                    + scff * (bix - bix1) * (biy2 - biy) * (biz2 - biz)
                                    + sfcc * (bix2 - bix) * (biy - biy1) * (biz - biz1)
                                    + sffc * (bix2 - bix) * (biy2 - biy) * (biz - biz1)
                                    + sccc * (bix - bix1) * (biy - biy1) * (biz - biz1)
                                    + scfc * (bix - bix1) * (biy2 - biy) * (biz - biz1)) * dxdydz;
                out[(size_t)(k - 1) + (size_t)nr * ((size_t)(j - 1) + (size_t)nzm * (i - 1))] = ans;
            }
}

}  // namespace

int tc_h5_load_continua(const tc_bou* cfg, const char* dir, double* qt, double* qr, double* qz, double* time) {
    if (!cfg || !qt || !qr || !qz) return fail(2000, "tc_h5_load_continua: null argument");
    const std::string master = join(dir, "continua_master.h5");
    std::vector<double> v;
    std::vector<uint64_t> d;
    std::string err;
    double s[6];
    const char* names[6] = {"nth", "nr", "nz", "time", "istr", "str"};
    for (int i = 0; i < 6; ++i) {
        if (!read_named(master, names[i], v, d, err)) return fail(2022, err);
        if (v.size() != 1) return fail(2022, std::string("master scalar '") + names[i] + "' is not a scalar");
        s[i] = v[0];
    }
    const int nthm = cfg->nthm, nzm = cfg->nzm, nrm = cfg->nrm, nr = nrm + 1;
    const int ntho = (int)s[0], nro = (int)s[1], nzo = (int)s[2], istro = (int)s[4];
    const double stro = s[5];
    // ReadFlowField.F90:64-116: another grid is interpolated (interp.F90)
    const bool other = ntho != nthm + 1 || nro != nr || nzo != nzm + 1 || istro != cfg->istr || stro != cfg->str;
    if (other) {
        if (nthm + 1 > ntho * 2 || nzm + 1 > nzo * 2 || nr > nro * 2)
            return fail(2024, "New grid resolution cannot be more than twice the old resolution");
        if (ntho < 3 || nzo < 3 || nro < 3) return fail(2024, "the continuation files hold a degenerate grid");
        std::vector<double> rc, rm;
        if (!gridnew(nro, cfg->rint, cfg->rext, istro, stro, rc, rm) || !gridnew(nr, cfg->rint, cfg->rext, cfg->istr, cfg->str, rc, rm))
            return fail(2024, "restart interpolation supports ISTR 0 and 6 only (interp.F90:267-274)");
    }
    const int fth = other ? ntho - 1 : nthm, fz = other ? nzo - 1 : nzm, fr = other ? nro : nr;
    const size_t halo = (size_t)(nthm + 2) * (nzm + 2) * nr;
    double* q[3] = {qt, qr, qz};
    std::vector<double> tmp;
    const char* files[3] = {"continua_qt.h5", "continua_qr.h5", "continua_qz.h5"};
    for (int c = 0; c < 3; ++c) {
        if (!read_named(join(dir, files[c]), "var", v, d, err)) return fail(2022, err);
        if (d.size() != 3 || d[0] != (uint64_t)fth || d[1] != (uint64_t)fz || d[2] != (uint64_t)fr)
            return fail(2024, std::string(files[c]) + ": dataset 'var' does not match continua_master.h5");
        if (other) {
            interp_field(v, ntho, nzo, nro, istro, stro, c + 1, *cfg, tmp);
            v.swap(tmp);
        }
        std::fill(q[c], q[c] + halo, 0.0);
        for (int i = 0; i < nthm; ++i)
            for (int j = 0; j < nzm; ++j)
                std::memcpy(&q[c][((size_t)(i + 1) * (nzm + 2) + (j + 1)) * nr], &v[((size_t)i * nzm + j) * nr],
                            sizeof(double) * nr);
    }
    // ReadFlowField.F90:144: IRESET = 1 starts the clock again at 0
    if (time) *time = cfg->ireset ? 0.0 : s[3];
    return 0;
}

int tc_h5_read_continua(tc_handle* h, const char* dir, double* time) {
    tc_bou b;
    if (!h || tc_get_bou(h, &b)) return hfail(h, 2000, "tc_h5_read_continua: null handle");
    const size_t halo = (size_t)(b.nthm + 2) * (b.nzm + 2) * (b.nrm + 1);
    std::vector<double> q[3];
    for (auto& a : q) a.resize(halo);
    double t = 0.0;
    if (int r = tc_h5_load_continua(&b, dir, q[0].data(), q[1].data(), q[2].data(), &t))
        return hfail(h, r, tc_last_error(nullptr));
    if (int r = tc_set_state(h, q[0].data(), q[1].data(), q[2].data(), nullptr)) return r;
    if (time) *time = t;
    // ReadFlowField.F90:149: TMAX counts from the time the run restarts at
    return tc_set_tmax(h, b.tmax + t);
}

int tc_h5_write_scalars(const char* path, int n, const char* const* names, const double* values, const int* is_int) {
    if (!path || n < 1 || !names || !values) return fail(2000, "tc_h5_write_scalars: bad argument");
    std::vector<WDataset> ds;
    for (int i = 0; i < n; ++i) {
        if (!names[i]) return fail(2000, "tc_h5_write_scalars: null name");
        ds.push_back(is_int && is_int[i] ? i32_dataset(names[i], (int32_t)std::lround(values[i]))
                                         : f64_dataset(names[i], {1}, &values[i]));
    }
    std::string err;
    if (!write_file(path, ds, err)) return fail(2021, err);
    return 0;
}

int tc_h5_write_grid_info(const tc_bou* cfg, const char* dir) {
    if (!cfg) return fail(2000, "tc_h5_write_grid_info: null argument");
    const int nthm = cfg->nthm, nzm = cfg->nzm, nrm = cfg->nrm, nr = nrm + 1;
    std::vector<double> rm(nr), rc(nr), tm(nthm), zm(nzm);
    if (tc_grid_array(cfg, TC_G_RM, rm.data(), nr) < 0 || tc_grid_array(cfg, TC_G_RC, rc.data(), nr) < 0)
        return fail(2001, "tc_h5_write_grid_info: invalid configuration");
    // CreateGrid.F90:61,72: tm(i) = (i - 1/2)/dxt, zm(j) = (j - 1/2)/dxz
    const double pi = 2.0 * std::asin(1.0);
    const double dxt = ((double)nthm * cfg->lamb) / (2.0 * pi), dxz = (double)nzm / cfg->alx3;
    for (int i = 0; i < nthm; ++i) tm[i] = ((double)i + 0.5) / dxt;
    for (int j = 0; j < nzm; ++j) zm[j] = ((double)j + 0.5) / dxz;
    std::string err;
    if (!write_file(join(dir, "cordin_info.h5"),
                    {f64_dataset("rm", {(uint64_t)nrm}, rm.data()), f64_dataset("rc", {(uint64_t)nr}, rc.data()),
                     f64_dataset("tm", {(uint64_t)nthm}, tm.data()), f64_dataset("zm", {(uint64_t)nzm}, zm.data())},
                    err))
        return fail(2021, err);
    return 0;
}

int tc_h5_write_stats(tc_handle* h, const char* dir, int readstats) {
    tc_bou b;
    if (!h || tc_get_bou(h, &b)) return hfail(h, 2000, "tc_h5_write_stats: null handle");
    static const char* const names[TC_ST_COUNT] = {
        "vt_mean", "vr_mean", "vz_mean", "wt_mean", "wr_mean", "wz_mean", "vt_rms", "vr_rms", "vz_rms",
        "wt_rms", "wr_rms", "wz_rms", "vtvr_mean", "vtvz_mean", "vrvz_mean", "pr_mean", "pr_rms", "disste"};
    const int nthm = b.nthm, nzm = b.nzm, nrm = b.nrm, nr = nrm + 1;
    const size_t ns = (size_t)nrm * nzm;
    std::vector<double> v(ns), old;
    std::vector<uint64_t> d;
    std::string err;
    for (int a = 0; a < TC_ST_COUNT; ++a) {
        if (int r = tc_get_stat(h, a, v.data())) return r;
        const std::string path = join(dir, (std::string(names[a]) + ".h5").c_str());
        if (readstats) {
            if (!read_named(path, names[a], old, d, err)) return hfail(h, 2022, err);
            if (old.size() != ns) return hfail(h, 2024, path + ": statistics of another grid");
            for (size_t t = 0; t < ns; ++t) v[t] = v[t] + old[t];
        }
        // HdfWriteSerialReal2D: Fortran (nrm, nzm) is the dataspace [nzm][nrm]
        if (!write_file(path, {f64_dataset(names[a], {(uint64_t)nzm, (uint64_t)nrm}, v.data())}, err))
            return hfail(h, 2021, err);
    }
    const std::string master = join(dir, "stafield_master.h5");
    int samples = tc_stat_samples(h);
    if (readstats) {
        if (!read_named(master, "averaging_time", old, d, err)) return hfail(h, 2022, err);
        samples += (int)old.at(0);
    }
    std::vector<double> rm(nr), tm(nthm), zm(nzm);
    if (tc_grid_array(&b, TC_G_RM, rm.data(), nr) < 0) return hfail(h, 2001, "tc_h5_write_stats: grid");
    const double pi = 2.0 * std::asin(1.0);
    const double dxt = ((double)nthm * b.lamb) / (2.0 * pi), dxz = (double)nzm / b.alx3;
    for (int i = 0; i < nthm; ++i) tm[i] = ((double)i + 0.5) / dxt;
    for (int j = 0; j < nzm; ++j) zm[j] = ((double)j + 0.5) / dxz;
    if (!write_file(master, {i32_dataset("averaging_time", samples), f64_dataset("R_cordin", {(uint64_t)nrm}, rm.data()),
                             f64_dataset("Th_cordin", {(uint64_t)nthm}, tm.data()),
                             f64_dataset("Z_cordin", {(uint64_t)nzm}, zm.data()),
                             f64_dataset("Reynolds Number", {1}, &b.ren), f64_dataset("R_Omega", {1}, &b.romeg)},
                    err))
        return hfail(h, 2021, err);
    return 0;
}

// ---- dumps of the output steps (main.F90:191-198) ---------------------------

namespace {

// itime = nint(1000 time + 0.005), written i8.8 (Dump*.F90)
std::string time_tag(double time) {
    char buf[32];
    std::snprintf(buf, sizeof buf, "%08ld", std::lround(1000.0 * time + 0.005));
    return buf;
}

struct HostState {
    tc_bou b;
    int nthm, nzm, nrm, nr;
    std::vector<double> q[3];
    size_t H(int k, int j, int i) const { return (size_t)(k - 1) + (size_t)nr * ((size_t)j + (size_t)(nzm + 2) * i); }
};

int load_state(tc_handle* h, HostState& s) {
    if (!h || tc_get_bou(h, &s.b)) return fail(2000, "null handle");
    s.nthm = s.b.nthm; s.nzm = s.b.nzm; s.nrm = s.b.nrm; s.nr = s.nrm + 1;
    for (auto& a : s.q) a.assign((size_t)(s.nthm + 2) * (s.nzm + 2) * s.nr, 0.0);
    return tc_get_state(h, s.q[0].data(), s.q[1].data(), s.q[2].data(), nullptr);
}

}  // namespace

int tc_h5_dump_flow_field(tc_handle* h, const char* dir, double time) {
    HostState s;
    if (int r = load_state(h, s)) return r;
    const std::string tag = time_tag(time);
    const char* pre[3] = {"qt_", "qr_", "qz_"};
    std::vector<double> in((size_t)s.nthm * s.nzm * s.nr);
    std::string err;
    for (int c = 0; c < 3; ++c) {   // HdfWriteRealHalo3D: q(1:nr, 1:nzm, 1:nthm)
        for (int i = 1; i <= s.nthm; ++i)
            for (int j = 1; j <= s.nzm; ++j)
                std::memcpy(&in[((size_t)(i - 1) * s.nzm + (j - 1)) * s.nr], &s.q[c][s.H(1, j, i)], sizeof(double) * s.nr);
        if (!write_file(join(dir, (pre[c] + tag + ".h5").c_str()),
                        {f64_dataset("var", {(uint64_t)s.nthm, (uint64_t)s.nzm, (uint64_t)s.nr}, in.data())}, err))
            return hfail(h, 2021, err);
    }
    const tc_bou& b = s.b;
    if (!write_file(join(dir, ("ms_" + tag + ".h5").c_str()),
                    {f64_dataset("time", {1}, &time), f64_dataset("rint", {1}, &b.rint), f64_dataset("rext", {1}, &b.rext),
                     i32_dataset("istr", b.istr), f64_dataset("str", {1}, &b.str), f64_dataset("alx3", {1}, &b.alx3),
                     f64_dataset("lamb", {1}, &b.lamb)},
                    err))
        return hfail(h, 2021, err);
    return 0;
}

int tc_h5_dump_rcuts(tc_handle* h, const char* dir, double time, const double* rslab, int nslab) {
    HostState s;
    if (int r = load_state(h, s)) return r;
    if (nslab < 0 || (nslab > 0 && !rslab)) return hfail(h, 2000, "tc_h5_dump_rcuts: bad slab list");
    if (nslab > 9) nslab = 9;   // InitDumpRCuts: at most 9 slabs
    std::vector<double> rm(s.nr), usrc(s.nr);
    if (tc_grid_array(&s.b, TC_G_RM, rm.data(), s.nr) < 0 || tc_grid_array(&s.b, TC_G_USRC, usrc.data(), s.nr) < 0)
        return hfail(h, 2001, "tc_h5_dump_rcuts: grid");
    const std::string tag = time_tag(time);
    std::vector<double> vt((size_t)s.nthm * s.nzm), vr(vt.size()), vz(vt.size());
    std::string err;
    for (int m = 1; m <= nslab; ++m) {
        // InitDumpRCuts: kslab = the k with rm(k-1) < rslab < rm(k), else 1
        int ks = 1;
        for (int k = 2; k <= s.nrm; ++k)
            if (rm[k - 1] > rslab[m - 1] && rm[k - 2] < rslab[m - 1]) ks = k;
        for (int i = 1; i <= s.nthm; ++i)
            for (int j = 1; j <= s.nzm; ++j) {
                const size_t o = (size_t)(i - 1) * s.nzm + (j - 1);   // Fortran (nzm, nthm): [nthm][nzm]
                vz[o] = s.q[2][s.H(ks, j, i)];
                vt[o] = s.q[0][s.H(ks, j, i)];
                vr[o] = (s.q[1][s.H(ks, j, i)] * usrc[ks - 1] + s.q[1][s.H(ks + 1, j, i)] * usrc[ks]) * 0.5;
            }
        const std::string sm = "slab" + std::to_string(m);
        const std::vector<uint64_t> dims{(uint64_t)s.nthm, (uint64_t)s.nzm};
        if (!write_file(join(dir, (sm + "vt_" + tag + ".h5").c_str()), {f64_dataset("vt", dims, vt.data())}, err) ||
            !write_file(join(dir, (sm + "vr_" + tag + ".h5").c_str()), {f64_dataset("vr", dims, vr.data())}, err) ||
            !write_file(join(dir, (sm + "vz_" + tag + ".h5").c_str()), {f64_dataset("vz", dims, vz.data())}, err))
            return hfail(h, 2021, err);
    }
    return 0;
}

int tc_h5_dump_thcuts(tc_handle* h, const char* dir, double time) {
    HostState s;
    if (int r = load_state(h, s)) return r;
    std::vector<double> usrc(s.nr);
    if (tc_grid_array(&s.b, TC_G_USRC, usrc.data(), s.nr) < 0) return hfail(h, 2001, "tc_h5_dump_thcuts: grid");
    const size_t ns = (size_t)s.nrm * s.nzm;
    std::vector<double> vt(ns), vr(ns), vz(ns);
    for (int j = 1; j <= s.nzm; ++j)        // the theta = 1 plane (DumpThCuts.F90:33-43)
        for (int k = 1; k <= s.nrm; ++k) {
            const size_t o = (size_t)(k - 1) + (size_t)s.nrm * (j - 1);
            vt[o] = s.q[0][s.H(k, j, 1)];
            vr[o] = s.q[1][s.H(k, j, 1)] * usrc[k - 1];
            vz[o] = s.q[2][s.H(k, j, 1)];
        }
    const std::string tag = time_tag(time);
    const std::vector<uint64_t> dims{(uint64_t)s.nzm, (uint64_t)s.nrm};
    std::string err;
    // DumpThCuts.F90:55-63 names the vr file slabvt_ too, so the vr dataset
    // replaces the vt one in that file, as in the reference
    if (!write_file(join(dir, ("slabvt_" + tag + ".h5").c_str()), {f64_dataset("vt", dims, vt.data())}, err) ||
        !write_file(join(dir, ("slabvt_" + tag + ".h5").c_str()), {f64_dataset("vr", dims, vr.data())}, err) ||
        !write_file(join(dir, ("slabvz_" + tag + ".h5").c_str()), {f64_dataset("vz", dims, vz.data())}, err))
        return hfail(h, 2021, err);
    return 0;
}

int tc_h5_dump_streamwise_avg(tc_handle* h, const char* dir, double time) {
    HostState s;
    if (int r = load_state(h, s)) return r;
    std::vector<double> usrc(s.nr);
    if (tc_grid_array(&s.b, TC_G_USRC, usrc.data(), s.nr) < 0) return hfail(h, 2001, "tc_h5_dump_streamwise_avg: grid");
    const size_t ns = (size_t)s.nrm * s.nzm;
    std::vector<double> vt(ns, 0.0), vr(ns, 0.0), vz(ns, 0.0);
    const double usnthm = 1.0 / (double)s.nthm;
    for (int i = 1; i <= s.nthm; ++i)       // DumpStreamwiseAvg.F90:33-42
        for (int j = 1; j <= s.nzm; ++j)
            for (int k = 1; k <= s.nrm; ++k) {
                const size_t o = (size_t)(k - 1) + (size_t)s.nrm * (j - 1);
                vt[o] = vt[o] + s.q[0][s.H(k, j, i)] * usnthm;
                vr[o] = vr[o] + s.q[1][s.H(k, j, i)] * usrc[k - 1] * usnthm;
                vz[o] = vz[o] + s.q[2][s.H(k, j, i)] * usnthm;
            }
    const std::string tag = time_tag(time);
    const std::vector<uint64_t> dims{(uint64_t)s.nzm, (uint64_t)s.nrm};
    std::string err;
    if (!write_file(join(dir, ("slabvt_ax_" + tag + ".h5").c_str()), {f64_dataset("vt", dims, vt.data())}, err) ||
        !write_file(join(dir, ("slabvr_ax_" + tag + ".h5").c_str()), {f64_dataset("vr", dims, vr.data())}, err) ||
        !write_file(join(dir, ("slabvz_ax_" + tag + ".h5").c_str()), {f64_dataset("vz", dims, vz.data())}, err))
        return hfail(h, 2021, err);
    return 0;
}
