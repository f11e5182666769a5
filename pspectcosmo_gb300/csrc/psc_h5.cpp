// psc_h5.cpp — minimal HDF5 writer (superblock 0, contiguous IEEE F64LE datasets).
// Field layouts follow the published HDF5 file format specification (sections II-IV:
// superblock, local heap, version-1 B-tree, symbol table node, version-1 object header
// and the dataspace, datatype, fill value, layout and symbol table messages).
#include "psc_h5.h"

#include <algorithm>
#include <cstring>

namespace psc {
namespace h5 {
namespace {

constexpr uint64_t kUndef = ~0ull;        // "undefined address"
constexpr uint64_t kFreeNull = 1;         // end of a local heap's free list
constexpr int kLeafK = 4;                 // group leaf node K: 2K = 8 entries per symbol table node
constexpr int kInternalK = 16;            // group internal node K: 2K = 32 children per B-tree node
constexpr size_t kSuperblock = 96;
constexpr size_t kEntry = 40;             // symbol table entry
constexpr size_t kSnod = 8 + 2 * kLeafK * kEntry;
constexpr size_t kBtree = 24 + (2 * kInternalK + 1) * 8 + 2 * kInternalK * 8;
constexpr size_t kHeapHeader = 32;

uint64_t align8(uint64_t x) { return (x + 7) & ~7ull; }

struct Buf {
    std::vector<unsigned char> b;
    explicit Buf(size_t n) : b(n, 0) {}
    void u8(size_t at, unsigned v) { b[at] = (unsigned char)v; }
    void le(size_t at, uint64_t v, int nbytes) {
        for (int i = 0; i < nbytes; ++i) b[at + i] = (unsigned char)(v >> (8 * i));
    }
    void bytes(size_t at, const void *p, size_t n) { std::memcpy(b.data() + at, p, n); }
};

// one object-header message: type, data size (multiple of 8), flags; returns the
// offset of its data
size_t msg(Buf &o, size_t at, unsigned type, unsigned size, unsigned flags) {
    o.le(at, type, 2);
    o.le(at + 2, size, 2);
    o.u8(at + 4, flags);
    return at + 8;
}

bool host_little_endian() {
    const uint16_t x = 1;
    unsigned char c;
    std::memcpy(&c, &x, 1);
    return c == 1;
}

}  // namespace

Writer::~Writer() {
    if (fp_) std::fclose(fp_);
}

int Writer::fail(const std::string &m) {
    err_ = m;
    if (fp_) std::fclose(fp_);
    fp_ = nullptr;
    return -1;
}

int Writer::open(const std::string &path, const std::vector<std::string> &names_in,
                 const std::vector<uint64_t> &dims) {
    return open(path, names_in, std::vector<std::vector<uint64_t>>(names_in.size(), dims));
}

int Writer::open(const std::string &path, const std::vector<std::string> &names_in,
                 const std::vector<std::vector<uint64_t>> &shapes) {
    if (!host_little_endian()) return fail("the HDF5 writer stores little-endian doubles from host memory");
    const size_t n = names_in.size();
    if (n == 0) return fail("no datasets");
    if (shapes.size() != n) return fail("one shape per dataset");
    for (const auto &dims : shapes)
        if (dims.empty() || dims.size() > 32) return fail("dataset rank must be 1..32");
    std::vector<std::string> names(n);
    for (size_t i = 0; i < n; ++i) {
        names[i] = (!names_in[i].empty() && names_in[i][0] == '/') ? names_in[i].substr(1) : names_in[i];
        if (names[i].empty() || names[i].find('/') != std::string::npos)
            return fail("dataset names must be non-empty and in the root group");
    }
    // symbol table nodes hold their entries sorted by name (strcmp order)
    std::vector<size_t> order(n);
    for (size_t i = 0; i < n; ++i) order[i] = i;
    std::sort(order.begin(), order.end(),
              [&](size_t x, size_t y) { return std::strcmp(names[x].c_str(), names[y].c_str()) < 0; });
    for (size_t i = 1; i < n; ++i)
        if (names[order[i]] == names[order[i - 1]]) return fail("duplicate dataset name " + names[order[i]]);
    const size_t per_snod = 2 * kLeafK;
    const size_t nsnod = (n + per_snod - 1) / per_snod;
    if (nsnod > (size_t)2 * kInternalK) return fail("too many datasets for one group node");

    // local heap data: "" at 0, the names at 8-byte aligned offsets, one free block
    std::vector<uint64_t> name_off(n);
    uint64_t heap_size = 8;
    for (size_t k = 0; k < n; ++k) {
        name_off[order[k]] = heap_size;
        heap_size += align8(names[order[k]].size() + 1);
    }
    const uint64_t free_off = heap_size;
    heap_size += 16;

    data_bytes_.assign(n, 0);
    std::vector<uint64_t> oh_size(n), oh_addr(n);
    const size_t type_sz = 24, fill_sz = 8, layout_sz = 24;
    for (size_t i = 0; i < n; ++i) {
        uint64_t elems = 1;
        for (uint64_t d : shapes[i]) {
            if (d == 0) return fail("zero-sized dimension");
            elems *= d;
        }
        data_bytes_[i] = elems * 8;
        const size_t space_sz = 8 + 8 * shapes[i].size();
        oh_size[i] = 16 + (8 + space_sz) + (8 + type_sz) + (8 + fill_sz) + (8 + layout_sz);
    }

    const uint64_t root_oh = kSuperblock;
    const uint64_t heap_hdr = root_oh + 16 + 8 + 16;
    const uint64_t heap_data = heap_hdr + kHeapHeader;
    const uint64_t btree = heap_data + heap_size;
    const uint64_t snod0 = btree + kBtree;
    const uint64_t oh0 = snod0 + nsnod * kSnod;
    uint64_t meta_end = oh0;
    for (size_t i = 0; i < n; ++i) {
        oh_addr[i] = meta_end;
        meta_end += oh_size[i];
    }
    data_addr_.assign(n, 0);
    uint64_t at_data = align8(meta_end);
    for (size_t i = 0; i < n; ++i) {
        data_addr_[i] = at_data;
        at_data += data_bytes_[i];
    }
    const uint64_t eof = at_data;

    Buf o((size_t)meta_end);
    // superblock version 0
    const unsigned char sig[8] = {0x89, 'H', 'D', 'F', '\r', '\n', 0x1a, '\n'};
    o.bytes(0, sig, 8);
    o.u8(13, 8);                 // size of offsets
    o.u8(14, 8);                 // size of lengths
    o.le(16, kLeafK, 2);
    o.le(18, kInternalK, 2);
    o.le(24, 0, 8);              // base address
    o.le(32, kUndef, 8);         // free-space info
    o.le(40, eof, 8);            // end of file
    o.le(48, kUndef, 8);         // driver information block
    o.le(56, 0, 8);              // root entry: link name offset ("")
    o.le(64, root_oh, 8);        //             object header
    o.le(72, 1, 4);              //             cache type 1: scratch pad holds the group's
    o.le(80, btree, 8);          //             B-tree and
    o.le(88, heap_hdr, 8);       //             local heap

    // root group object header (version 1) with its symbol table message
    o.u8(root_oh, 1);
    o.le(root_oh + 2, 1, 2);     // one message
    o.le(root_oh + 4, 1, 4);     // reference count
    o.le(root_oh + 8, 8 + 16, 4);
    size_t d = msg(o, root_oh + 16, 0x0011, 16, 1);
    o.le(d, btree, 8);
    o.le(d + 8, heap_hdr, 8);

    // local heap
    o.bytes(heap_hdr, "HEAP", 4);
    o.le(heap_hdr + 8, heap_size, 8);
    o.le(heap_hdr + 16, free_off, 8);
    o.le(heap_hdr + 24, heap_data, 8);
    for (size_t i = 0; i < n; ++i) o.bytes(heap_data + name_off[i], names[i].c_str(), names[i].size() + 1);
    o.le(heap_data + free_off, kFreeNull, 8);
    o.le(heap_data + free_off + 8, 16, 8);

    // B-tree leaf (node type 0 = group): key 0 = "", child i = symbol table node i,
    // key i+1 = the last (largest) name of child i
    o.bytes(btree, "TREE", 4);
    o.le(btree + 6, nsnod, 2);
    o.le(btree + 8, kUndef, 8);
    o.le(btree + 16, kUndef, 8);
    size_t kp = btree + 24;
    o.le(kp, 0, 8);
    for (size_t s = 0; s < nsnod; ++s) {
        const size_t last = std::min(n, (s + 1) * per_snod) - 1;
        o.le(kp + 8, snod0 + s * kSnod, 8);
        o.le(kp + 16, name_off[order[last]], 8);
        kp += 16;
    }

    // symbol table nodes
    for (size_t s = 0; s < nsnod; ++s) {
        const size_t at = snod0 + s * kSnod;
        const size_t first = s * per_snod, cnt = std::min(n, first + per_snod) - first;
        o.bytes(at, "SNOD", 4);
        o.u8(at + 4, 1);
        o.le(at + 6, cnt, 2);
        for (size_t e = 0; e < cnt; ++e) {
            const size_t i = order[first + e], ep = at + 8 + e * kEntry;
            o.le(ep, name_off[i], 8);
            o.le(ep + 8, oh_addr[i], 8);   // cache type 0, empty scratch pad
        }
    }

    // dataset object headers (version 1)
    for (size_t i = 0; i < n; ++i) {
        const size_t at = oh_addr[i];
        const std::vector<uint64_t> &dims = shapes[i];
        const size_t rank = dims.size(), space_sz = 8 + 8 * rank;
        o.u8(at, 1);
        o.le(at + 2, 4, 2);
        o.le(at + 4, 1, 4);
        o.le(at + 8, oh_size[i] - 16, 4);
        // dataspace, version 1: rank, no maximum dimensions
        d = msg(o, at + 16, 0x0001, (unsigned)space_sz, 0);
        o.u8(d, 1);
        o.u8(d + 1, (unsigned)rank);
        for (size_t r = 0; r < rank; ++r) o.le(d + 8 + 8 * r, dims[r], 8);
        // datatype, version 1, class 1 (floating point): little endian, implied
        // mantissa msb, sign bit 63; 8 bytes; offset 0, precision 64, exponent at 52
        // (11 bits), mantissa at 0 (52 bits), bias 1023
        d = msg(o, d + space_sz, 0x0003, (unsigned)type_sz, 1);
        o.u8(d, 0x11);
        o.u8(d + 1, 0x20);
        o.u8(d + 2, 63);
        o.le(d + 4, 8, 4);
        o.le(d + 8, 0, 2);
        o.le(d + 10, 64, 2);
        o.u8(d + 12, 52);
        o.u8(d + 13, 11);
        o.u8(d + 14, 0);
        o.u8(d + 15, 52);
        o.le(d + 16, 1023, 4);
        // fill value, version 1: allocation late, write if set, defined, default (size 0)
        d = msg(o, d + type_sz, 0x0005, (unsigned)fill_sz, 1);
        o.u8(d, 1);
        o.u8(d + 1, 2);
        o.u8(d + 2, 2);
        o.u8(d + 3, 1);
        // data layout, version 3: contiguous at data_addr_, data_bytes_ long
        d = msg(o, d + fill_sz, 0x0008, (unsigned)layout_sz, 1);
        o.u8(d, 3);
        o.u8(d + 1, 1);
        o.le(d + 2, data_addr_[i], 8);
        o.le(d + 10, data_bytes_[i], 8);
    }

    fp_ = std::fopen(path.c_str(), "wb");
    if (!fp_) return fail("cannot create " + path);
    if (std::fwrite(o.b.data(), 1, o.b.size(), fp_) != o.b.size()) return fail("write failed: " + path);
    // the file is eof bytes long even before the data are written
    const unsigned char z = 0;
    if (fseeko(fp_, (off_t)(eof - 1), SEEK_SET) != 0 || std::fwrite(&z, 1, 1, fp_) != 1)
        return fail("cannot extend " + path);
    return 0;
}

int Writer::write(int i, const double *data) {
    if (!fp_) return fail("file not open");
    if (i < 0 || (size_t)i >= data_addr_.size()) return fail("no such dataset");
    if (fseeko(fp_, (off_t)data_addr_[i], SEEK_SET) != 0) return fail("seek failed");
    const size_t cnt = (size_t)(data_bytes_[i] / 8);
    if (std::fwrite(data, 8, cnt, fp_) != cnt) return fail("write failed");
    return 0;
}

int Writer::close() {
    if (!fp_) return 0;
    const int rc = std::fclose(fp_);
    fp_ = nullptr;
    if (rc != 0) return fail("close failed");
    return 0;
}

Reader::~Reader() {
    if (fp_) std::fclose(fp_);
}

int Reader::fail(const std::string &m) {
    err_ = m;
    return -1;
}

int Reader::get(uint64_t addr, void *dst, size_t n) {
    if (addr > eof_ || n > eof_ - addr) return fail("structure outside the file");
    if (fseeko(fp_, (off_t)addr, SEEK_SET) != 0 || std::fread(dst, 1, n, fp_) != n) return fail("read failed");
    return 0;
}

namespace {
uint64_t rd(const unsigned char *p, int nbytes) {
    uint64_t v = 0;
    for (int i = nbytes - 1; i >= 0; --i) v = (v << 8) | p[i];
    return v;
}
}  // namespace

int Reader::open(const std::string &path) {
    if (!host_little_endian()) return fail("the HDF5 reader fills little-endian doubles into host memory");
    fp_ = std::fopen(path.c_str(), "rb");
    if (!fp_) return fail("cannot open " + path);
    if (fseeko(fp_, 0, SEEK_END) != 0) return fail("seek failed");
    eof_ = (uint64_t)ftello(fp_);
    unsigned char sb[kSuperblock];
    if (get(0, sb, sizeof sb)) return -1;
    const unsigned char sig[8] = {0x89, 'H', 'D', 'F', '\r', '\n', 0x1a, '\n'};
    if (std::memcmp(sb, sig, 8) != 0) return fail("not an HDF5 file (at offset 0)");
    if (sb[8] != 0 || sb[13] != 8 || sb[14] != 8) return fail("unsupported HDF5 superblock");
    if (rd(sb + 24, 8) != 0) return fail("unsupported base address");
    const uint64_t btree = rd(sb + 80, 8), heap = rd(sb + 88, 8);
    if (rd(sb + 72, 4) != 1) return fail("root group without a cached symbol table");
    unsigned char hh[kHeapHeader];
    if (get(heap, hh, sizeof hh)) return -1;
    if (std::memcmp(hh, "HEAP", 4) != 0) return fail("bad local heap");
    const uint64_t heap_size = rd(hh + 8, 8), heap_data = rd(hh + 24, 8);
    if (heap_size > (1u << 24)) return fail("local heap too large");
    std::vector<unsigned char> names(heap_size + 1, 0);
    if (get(heap_data, names.data(), heap_size)) return -1;
    std::vector<unsigned char> bt(kBtree);
    if (get(btree, bt.data(), bt.size())) return -1;
    if (std::memcmp(bt.data(), "TREE", 4) != 0 || bt[4] != 0 || bt[5] != 0)
        return fail("unsupported group B-tree (only one leaf node)");
    const unsigned used = (unsigned)rd(bt.data() + 6, 2);
    if (used > 2u * kInternalK) return fail("bad B-tree node");
    for (unsigned c = 0; c < used; ++c) {
        const uint64_t snod = rd(bt.data() + 24 + 8 + 16 * c, 8);
        std::vector<unsigned char> sn(kSnod);
        if (get(snod, sn.data(), sn.size())) return -1;
        if (std::memcmp(sn.data(), "SNOD", 4) != 0) return fail("bad symbol table node");
        const unsigned nsym = (unsigned)rd(sn.data() + 6, 2);
        if (nsym > 2u * kLeafK) return fail("bad symbol table node");
        for (unsigned e = 0; e < nsym; ++e) {
            const unsigned char *ep = sn.data() + 8 + e * kEntry;
            const uint64_t off = rd(ep, 8);
            if (off >= heap_size) return fail("bad link name");
            links_.emplace_back(std::string(reinterpret_cast<const char *>(names.data() + off)), rd(ep + 8, 8));
        }
    }
    return 0;
}

int Reader::dataset(const std::string &name_in, Dset *d) {
    const std::string name = (!name_in.empty() && name_in[0] == '/') ? name_in.substr(1) : name_in;
    uint64_t oh = 0;
    bool found = false;
    for (const auto &l : links_)
        if (l.first == name) {
            oh = l.second;
            found = true;
        }
    if (!found) return fail("no dataset " + name);
    unsigned char pre[16];
    if (get(oh, pre, sizeof pre)) return -1;
    if (pre[0] != 1) return fail("unsupported object header");
    const unsigned nmsg = (unsigned)rd(pre + 2, 2);
    const uint64_t size = rd(pre + 8, 4);
    if (size > 4096) return fail("object header too large");
    std::vector<unsigned char> m(size);
    if (get(oh + 16, m.data(), m.size())) return -1;
    bool space = false, type = false, layout = false;
    size_t q = 0;
    for (unsigned i = 0; i < nmsg && q + 8 <= m.size(); ++i) {
        const unsigned mt = (unsigned)rd(&m[q], 2), ms = (unsigned)rd(&m[q + 2], 2);
        if (q + 8 + ms > m.size()) return fail("bad object header message");
        const unsigned char *b = &m[q + 8];
        if (mt == 0x0001) {
            if (b[0] != 1 || ms < 8u + 8u * b[1]) return fail("unsupported dataspace");
            d->dims.clear();
            for (int r = 0; r < b[1]; ++r) d->dims.push_back(rd(b + 8 + 8 * r, 8));
            space = true;
        } else if (mt == 0x0003) {
            if ((b[0] & 0x0f) != 1 || (b[1] & 1) != 0 || rd(b + 4, 4) != 8) return fail("dataset is not F64LE");
            type = true;
        } else if (mt == 0x0008) {
            if (b[0] != 3 || b[1] != 1) return fail("dataset is not contiguous");
            d->addr = rd(b + 2, 8);
            d->bytes = rd(b + 10, 8);
            layout = true;
        }
        q += 8 + ms;
    }
    if (!space || !type || !layout) return fail("incomplete dataset header: " + name);
    uint64_t count = 1;
    for (uint64_t x : d->dims) count *= x;
    if (count * 8 != d->bytes) return fail("dataset size disagrees with its shape: " + name);
    return 0;
}

int Reader::shape(const std::string &name, std::vector<uint64_t> *dims) {
    Dset d;
    if (dataset(name, &d)) return -1;
    *dims = d.dims;
    return 0;
}

int Reader::read(const std::string &name, double *out, size_t count) {
    Dset d;
    if (dataset(name, &d)) return -1;
    if (d.bytes != (uint64_t)count * 8) return fail("dataset " + name + " has another size");
    return get(d.addr, out, (size_t)d.bytes);
}

}  // namespace h5
}  // namespace psc
