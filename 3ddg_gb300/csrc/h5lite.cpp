// Library-free HDF5 writer; see h5lite.h.  Field layouts follow the HDF5 file
// format specification (superblock v0, object header v1, dataspace message
// v1, datatype message v1 class 1, fill value message v2, data layout message
// v3, v1 group B-tree, local heap, symbol table node).
#include "h5lite.h"

#include <algorithm>
#include <cstdio>
#include <cstring>

namespace dg {

namespace {

constexpr uint64_t UNDEF = ~0ull;
constexpr int LEAF_K = 4;       // group leaf node K: a symbol node holds 2K entries
constexpr int INTERNAL_K = 16;  // group internal node K: a B-tree node has room for 2K children
constexpr size_t OH_CHUNK_MIN = 256;

struct Buf {
    std::vector<uint8_t> b;
    void u8(uint8_t v) { b.push_back(v); }
    void u16(uint16_t v) { for (int i = 0; i < 2; i++) b.push_back((uint8_t)(v >> (8 * i))); }
    void u32(uint32_t v) { for (int i = 0; i < 4; i++) b.push_back((uint8_t)(v >> (8 * i))); }
    void u64(uint64_t v) { for (int i = 0; i < 8; i++) b.push_back((uint8_t)(v >> (8 * i))); }
    void bytes(const void* p, size_t n) { const uint8_t* c = (const uint8_t*)p; b.insert(b.end(), c, c + n); }
    void zeros(size_t n) { b.insert(b.end(), n, 0); }
    void pad8() { while (b.size() % 8) b.push_back(0); }
    size_t size() const { return b.size(); }
};

inline size_t pad8(size_t n) { return (n + 7) / 8 * 8; }

// A header message: type, data padded to a multiple of 8.
struct Msg {
    uint16_t type;
    Buf data;
};

void put_msg(Buf& out, const Msg& m)
{
    out.u16(m.type);
    out.u16((uint16_t)pad8(m.data.size()));
    out.u8(0);  // flags
    out.zeros(3);
    out.bytes(m.data.b.data(), m.data.size());
    out.zeros(pad8(m.data.size()) - m.data.size());
}

// Version-1 object header with the given messages, its chunk padded with a
// NIL message to at least OH_CHUNK_MIN bytes.
Buf object_header(const std::vector<Msg>& msgs)
{
    size_t chunk = 0;
    for (const Msg& m : msgs) chunk += 8 + pad8(m.data.size());
    size_t nil = 0;
    int nmsg = (int)msgs.size();
    if (chunk < OH_CHUNK_MIN) {
        nil = OH_CHUNK_MIN - chunk;  // >= 8 because both are multiples of 8
        chunk = OH_CHUNK_MIN;
        nmsg++;
    }
    Buf h;
    h.u8(1);   // version
    h.u8(0);   // reserved
    h.u16((uint16_t)nmsg);
    h.u32(1);  // reference count
    h.u32((uint32_t)chunk);
    h.zeros(4);  // alignment of the message area
    for (const Msg& m : msgs) put_msg(h, m);
    if (nil) {
        h.u16(0);
        h.u16((uint16_t)(nil - 8));
        h.u8(0);
        h.zeros(3);
        h.zeros(nil - 8);
    }
    return h;
}

Msg dataspace_msg(const std::vector<uint64_t>& dims)
{
    Msg m{0x0001, {}};
    m.data.u8(1);  // version
    m.data.u8((uint8_t)dims.size());
    m.data.u8(0);  // flags: no maximum dimensions
    m.data.u8(0);
    m.data.u32(0);
    for (uint64_t d : dims) m.data.u64(d);
    return m;
}

Msg f64_type_msg()
{
    Msg m{0x0003, {}};
    m.data.u8(0x11);  // version 1, class 1 (floating point)
    m.data.u8(0x20);  // little-endian, no padding, implied mantissa MSB
    m.data.u8(63);    // sign bit location
    m.data.u8(0);
    m.data.u32(8);    // size in bytes
    m.data.u16(0);    // bit offset
    m.data.u16(64);   // bit precision
    m.data.u8(52);    // exponent location
    m.data.u8(11);    // exponent size
    m.data.u8(0);     // mantissa location
    m.data.u8(52);    // mantissa size
    m.data.u32(1023); // exponent bias
    return m;
}

Msg fill_msg()
{
    Msg m{0x0005, {}};
    m.data.u8(2);  // version
    m.data.u8(1);  // space allocation time: early
    m.data.u8(2);  // fill value write time: if set by user
    m.data.u8(0);  // fill value not defined
    return m;
}

Msg layout_msg(uint64_t addr, uint64_t size)
{
    Msg m{0x0008, {}};
    m.data.u8(3);  // version
    m.data.u8(1);  // contiguous
    m.data.u64(addr);
    m.data.u64(size);
    return m;
}

}  // namespace

int h5_write(const std::string& path, const std::vector<H5Dataset>& sets_in)
{
    if (sets_in.empty() || sets_in.size() > 2 * LEAF_K) return -1;
    std::vector<H5Dataset> sets = sets_in;
    std::sort(sets.begin(), sets.end(), [](const H5Dataset& a, const H5Dataset& b) { return a.name < b.name; });

    // Local heap data: "" at 0, then each name, each padded to 8 bytes.
    Buf heap_data;
    heap_data.u8(0);
    heap_data.pad8();
    std::vector<uint64_t> name_off;
    for (const H5Dataset& s : sets) {
        name_off.push_back(heap_data.size());
        heap_data.bytes(s.name.c_str(), s.name.size() + 1);
        heap_data.pad8();
    }

    const uint64_t SB = 0, SB_SIZE = 96;
    const uint64_t ROOT_OH = SB + SB_SIZE;
    const uint64_t ROOT_OH_SIZE = 16 + OH_CHUNK_MIN;
    const uint64_t BTREE = ROOT_OH + ROOT_OH_SIZE;
    const uint64_t BTREE_SIZE = 24 + (2 * INTERNAL_K + 1) * 8 + 2 * INTERNAL_K * 8;
    const uint64_t HEAP = BTREE + BTREE_SIZE;
    const uint64_t HEAP_HDR = 32;
    const uint64_t HEAP_DATA = HEAP + HEAP_HDR;
    const uint64_t SNOD = HEAP_DATA + heap_data.size();
    const uint64_t SNOD_SIZE = 8 + 2 * LEAF_K * 40;

    // Dataset object headers; their sizes do not depend on the data address.
    std::vector<uint64_t> oh_addr(sets.size()), data_addr(sets.size()), data_size(sets.size());
    uint64_t cursor = SNOD + SNOD_SIZE;
    std::vector<Buf> ohs(sets.size());
    for (size_t i = 0; i < sets.size(); i++) {
        uint64_t n = 1;
        for (uint64_t d : sets[i].dims) n *= d;
        data_size[i] = n * 8;
        std::vector<Msg> probe = {dataspace_msg(sets[i].dims), f64_type_msg(), fill_msg(), layout_msg(0, 0)};
        oh_addr[i] = cursor;
        cursor += object_header(probe).size();
    }
    for (size_t i = 0; i < sets.size(); i++) {
        data_addr[i] = cursor;
        cursor += pad8(data_size[i]);
        ohs[i] = object_header({dataspace_msg(sets[i].dims), f64_type_msg(), fill_msg(),
                                layout_msg(data_addr[i], data_size[i])});
    }
    const uint64_t EOFA = cursor;

    Buf f;
    // Superblock v0
    const uint8_t sig[8] = {0x89, 'H', 'D', 'F', '\r', '\n', 0x1a, '\n'};
    f.bytes(sig, 8);
    f.u8(0);  // superblock version
    f.u8(0);  // free-space version
    f.u8(0);  // root group symbol table entry version
    f.u8(0);
    f.u8(0);  // shared header message format version
    f.u8(8);  // size of offsets
    f.u8(8);  // size of lengths
    f.u8(0);
    f.u16(LEAF_K);
    f.u16(INTERNAL_K);
    f.u32(0);  // file consistency flags
    f.u64(0);  // base address
    f.u64(UNDEF);  // free-space info
    f.u64(EOFA);
    f.u64(UNDEF);  // driver information block
    // root group symbol table entry
    f.u64(0);
    f.u64(ROOT_OH);
    f.u32(1);  // cache type: B-tree and heap addresses in the scratch pad
    f.u32(0);
    f.u64(BTREE);
    f.u64(HEAP);
    // Root group object header: symbol table message
    {
        Msg st{0x0011, {}};
        st.data.u64(BTREE);
        st.data.u64(HEAP);
        Buf h = object_header({st});
        f.bytes(h.b.data(), h.size());
    }
    // v1 B-tree node (group), one child: the symbol table node
    f.bytes("TREE", 4);
    f.u8(0);   // node type: group
    f.u8(0);   // level: leaf
    f.u16(1);  // entries used
    f.u64(UNDEF);
    f.u64(UNDEF);
    f.u64(0);                 // key 0: the empty name
    f.u64(SNOD);              // child 0
    f.u64(name_off.back());   // key 1: the largest name in child 0
    f.zeros(BTREE_SIZE - 24 - 3 * 8);
    // Local heap
    f.bytes("HEAP", 4);
    f.u8(0);
    f.zeros(3);
    f.u64(heap_data.size());
    f.u64(1);  // free-list head: the on-disk "no free block" value
    f.u64(HEAP_DATA);
    f.bytes(heap_data.b.data(), heap_data.size());
    // Symbol table node
    f.bytes("SNOD", 4);
    f.u8(1);
    f.u8(0);
    f.u16((uint16_t)sets.size());
    for (size_t i = 0; i < 2 * LEAF_K; i++) {
        if (i < sets.size()) {
            f.u64(name_off[i]);
            f.u64(oh_addr[i]);
            f.u32(0);  // no cache
            f.u32(0);
            f.zeros(16);
        } else {
            f.zeros(40);
        }
    }
    for (size_t i = 0; i < sets.size(); i++) f.bytes(ohs[i].b.data(), ohs[i].size());
    if (f.size() != data_addr[0]) return -1;  // layout bookkeeping error

    FILE* fp = std::fopen(path.c_str(), "wb");
    if (!fp) return -1;
    bool ok = std::fwrite(f.b.data(), 1, f.size(), fp) == f.size();
    for (size_t i = 0; i < sets.size() && ok; i++) {
        ok = std::fwrite(sets[i].data, 1, data_size[i], fp) == data_size[i];
        static const uint8_t z[8] = {0};
        size_t pad = pad8(data_size[i]) - data_size[i];
        if (ok && pad) ok = std::fwrite(z, 1, pad, fp) == pad;
    }
    ok = (std::fclose(fp) == 0) && ok;
    return ok ? 0 : -1;
}

}  // namespace dg
