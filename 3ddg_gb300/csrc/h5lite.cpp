// Library-free HDF5 writer; see h5lite.h.  Field layouts follow the HDF5 file
// format specification (superblock v0, object header v1, dataspace message
// v1, datatype message v1 class 1, fill value message v2, data layout message
// v3, v1 group B-tree, local heap, symbol table node).
#include "h5lite.h"

#include <algorithm>
#include <cstdio>
#include <cstring>
#include <new>

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

// ---------------------------------------------------------------------------
// Reader.  Every field read is bounds-checked against the file; a malformed
// file gives an error code, never an out-of-range access.
// ---------------------------------------------------------------------------
namespace dg {

namespace {

struct H5Error {
    int code;
    std::string msg;
};

struct Reader {
    std::vector<uint8_t> b;
    void need(uint64_t off, uint64_t n, int code, const char* what) const
    {
        if (off > b.size() || n > b.size() - off) throw H5Error{code, std::string("truncated ") + what};
    }
    uint64_t uN(uint64_t off, int n, int code, const char* what) const
    {
        need(off, (uint64_t)n, code, what);
        uint64_t v = 0;
        for (int i = n - 1; i >= 0; i--) v = (v << 8) | b[off + i];
        return v;
    }
    uint64_t u64(uint64_t off, int code, const char* what) const { return uN(off, 8, code, what); }
    uint32_t u32(uint64_t off, int code, const char* what) const { return (uint32_t)uN(off, 4, code, what); }
    uint16_t u16(uint64_t off, int code, const char* what) const { return (uint16_t)uN(off, 2, code, what); }
    uint8_t u8(uint64_t off, int code, const char* what) const { return (uint8_t)uN(off, 1, code, what); }
};

struct MsgRef {
    uint16_t type;
    uint64_t off, size;
};

// Messages of a version-1 object header, following continuation messages.
std::vector<MsgRef> header_messages(const Reader& r, uint64_t base, uint64_t addr, int code)
{
    if (r.u8(base + addr, code, "object header") != 1)
        throw H5Error{code, "object header version is not 1"};
    const uint16_t nmsg = r.u16(base + addr + 2, code, "object header");
    const uint32_t size = r.u32(base + addr + 8, code, "object header");
    std::vector<std::pair<uint64_t, uint64_t>> blocks{{base + addr + 16, size}};
    std::vector<MsgRef> out;
    for (size_t bi = 0; bi < blocks.size() && out.size() < nmsg; bi++) {
        if (bi > 64) throw H5Error{code, "too many object header continuation blocks"};
        uint64_t p = blocks[bi].first;
        const uint64_t end = p + blocks[bi].second;
        r.need(blocks[bi].first, blocks[bi].second, code, "object header block");
        while (p + 8 <= end && out.size() < nmsg) {
            const uint16_t type = r.u16(p, code, "message");
            const uint16_t msize = r.u16(p + 2, code, "message");
            if (p + 8 + msize > end) throw H5Error{code, "message overruns its header block"};
            out.push_back({type, p + 8, msize});
            if (type == 0x0010) {
                blocks.push_back({base + r.u64(p + 8, code, "continuation"), r.u64(p + 16, code, "continuation")});
            }
            p += 8 + msize;
        }
    }
    return out;
}

void walk_group_btree(const Reader& r, uint64_t base, uint64_t node, uint64_t heap_data, int depth,
                      std::vector<std::pair<std::string, uint64_t>>& out)
{
    if (depth > 32) throw H5Error{-1, "group B-tree too deep"};
    r.need(base + node, 24, -1, "B-tree node");
    if (std::memcmp(&r.b[base + node], "TREE", 4) != 0) throw H5Error{-1, "bad B-tree node signature"};
    if (r.u8(base + node + 4, -1, "B-tree") != 0) throw H5Error{-1, "not a group B-tree"};
    const int level = r.u8(base + node + 5, -1, "B-tree");
    const int used = r.u16(base + node + 6, -1, "B-tree");
    uint64_t p = base + node + 24 + 8;  // past key 0
    for (int i = 0; i < used; i++, p += 16) {
        const uint64_t child = r.u64(p, -1, "B-tree child");
        if (level > 0) {
            walk_group_btree(r, base, child, heap_data, depth + 1, out);
            continue;
        }
        r.need(base + child, 8, -1, "symbol table node");
        if (std::memcmp(&r.b[base + child], "SNOD", 4) != 0) throw H5Error{-1, "bad symbol table node signature"};
        const int nsym = r.u16(base + child + 6, -1, "symbol table node");
        for (int k = 0; k < nsym; k++) {
            const uint64_t e = base + child + 8 + 40ull * k;
            const uint64_t noff = r.u64(e, -1, "symbol entry");
            const uint64_t oh = r.u64(e + 8, -1, "symbol entry");
            uint64_t s = base + heap_data + noff, q = s;
            while (true) {
                if (r.u8(q, -1, "link name") == 0) break;
                q++;
            }
            out.push_back({std::string((const char*)&r.b[s], q - s), oh});
        }
    }
}

double to_double(const uint8_t* p, int cls, int size, bool be, bool sgn)
{
    uint8_t t[8];
    for (int i = 0; i < size; i++) t[i] = be ? p[size - 1 - i] : p[i];
    if (cls == 1) {
        if (size == 8) {
            double d;
            std::memcpy(&d, t, 8);
            return d;
        }
        float f;
        std::memcpy(&f, t, 4);
        return (double)f;
    }
    uint64_t v = 0;
    for (int i = size - 1; i >= 0; i--) v = (v << 8) | t[i];
    if (sgn && size < 8 && (v >> (8 * size - 1)) & 1) v |= ~0ull << (8 * size);
    return sgn ? (double)(int64_t)v : (double)v;
}

}  // namespace

int h5_read(const std::string& path, const std::string& name, std::vector<uint64_t>& dims,
            std::vector<double>& data, int* type_class, std::string* why)
{
    try {
        Reader r;
        {
            FILE* fp = std::fopen(path.c_str(), "rb");
            if (!fp) throw H5Error{-1, "cannot open " + path};
            std::fseek(fp, 0, SEEK_END);
            const long n = std::ftell(fp);
            std::fseek(fp, 0, SEEK_SET);
            if (n < 0) {
                std::fclose(fp);
                throw H5Error{-1, "cannot size " + path};
            }
            r.b.resize((size_t)n);
            const bool ok = std::fread(r.b.data(), 1, r.b.size(), fp) == r.b.size();
            std::fclose(fp);
            if (!ok) throw H5Error{-1, "cannot read " + path};
        }
        // The superblock sits at 0, 512, 1024, 2048, ...
        static const uint8_t sig[8] = {0x89, 'H', 'D', 'F', '\r', '\n', 0x1a, '\n'};
        uint64_t sb = UNDEF;
        for (uint64_t o = 0; o + 8 <= r.b.size(); o = o ? 2 * o : 512)
            if (std::memcmp(&r.b[o], sig, 8) == 0) {
                sb = o;
                break;
            }
        if (sb == UNDEF) throw H5Error{-1, "not an HDF5 file"};
        const int ver = r.u8(sb + 8, -1, "superblock");
        if (ver > 1) throw H5Error{-1, "superblock version " + std::to_string(ver) + " is not supported"};
        if (r.u8(sb + 13, -1, "superblock") != 8 || r.u8(sb + 14, -1, "superblock") != 8)
            throw H5Error{-1, "only 8-byte offsets and lengths are supported"};
        const uint64_t fields = sb + 24 + (ver == 1 ? 4 : 0);
        const uint64_t base = r.u64(fields, -1, "superblock");
        const uint64_t root_oh = r.u64(fields + 32 + 8, -1, "root symbol table entry");

        uint64_t btree = UNDEF, heap = UNDEF;
        for (const MsgRef& m : header_messages(r, base, root_oh, -1))
            if (m.type == 0x0011) {
                btree = r.u64(m.off, -1, "symbol table message");
                heap = r.u64(m.off + 8, -1, "symbol table message");
            }
        if (btree == UNDEF) throw H5Error{-1, "root group has no symbol table (new-style groups are not supported)"};
        r.need(base + heap, 32, -1, "local heap");
        if (std::memcmp(&r.b[base + heap], "HEAP", 4) != 0) throw H5Error{-1, "bad local heap signature"};
        const uint64_t heap_data = r.u64(base + heap + 24, -1, "local heap");
        std::vector<std::pair<std::string, uint64_t>> entries;
        walk_group_btree(r, base, btree, heap_data, 0, entries);
        uint64_t oh = UNDEF;
        for (auto& e : entries)
            if (e.first == name) oh = e.second;
        if (oh == UNDEF) throw H5Error{-2, "no dataset named '" + name + "'"};

        bool have_space = false, have_type = false, have_layout = false;
        int cls = -1, size = 0;
        bool be = false, sgn = false;
        uint64_t daddr = UNDEF, dsize = 0, compact_off = UNDEF;
        dims.clear();
        for (const MsgRef& m : header_messages(r, base, oh, -2)) {
            if (m.type == 0x0001) {
                const int v = r.u8(m.off, -3, "dataspace"), nd = r.u8(m.off + 1, -3, "dataspace");
                if (v == 2 && r.u8(m.off + 3, -3, "dataspace") == 2) throw H5Error{-3, "null dataspace"};
                if (nd > 32) throw H5Error{-3, "dataspace rank above 32"};
                const uint64_t q = m.off + (v == 1 ? 8 : 4);
                for (int i = 0; i < nd; i++) dims.push_back(r.u64(q + 8ull * i, -3, "dataspace"));
                have_space = true;
            } else if (m.type == 0x0003) {
                const uint8_t c0 = r.u8(m.off, -4, "datatype"), c1 = r.u8(m.off + 1, -4, "datatype");
                cls = c0 & 0x0F;
                size = (int)r.u32(m.off + 4, -4, "datatype");
                be = (c1 & 1) != 0;
                sgn = ((c1 >> 3) & 1) != 0;
                if (cls == 1 && (size == 4 || size == 8) && !(c1 & 0x40)) {
                    // IEEE single or double (not VAX order)
                } else if (cls == 0 && size >= 1 && size <= 8) {
                } else {
                    throw H5Error{-4, "datatype class " + std::to_string(cls) + " size " + std::to_string(size) +
                                          " is not an integer or IEEE float"};
                }
                have_type = true;
            } else if (m.type == 0x0008) {
                const int v = r.u8(m.off, -2, "layout");
                if (v == 3) {
                    const int lc = r.u8(m.off + 1, -2, "layout");
                    if (lc == 1) {
                        daddr = r.u64(m.off + 2, -2, "layout");
                        dsize = r.u64(m.off + 10, -2, "layout");
                    } else if (lc == 0) {
                        dsize = r.u16(m.off + 2, -2, "layout");
                        compact_off = m.off + 4;
                    } else {
                        throw H5Error{-2, "chunked or virtual layout is not supported"};
                    }
                } else if (v == 1 || v == 2) {
                    const int nd = r.u8(m.off + 1, -2, "layout"), lc = r.u8(m.off + 2, -2, "layout");
                    if (lc == 1) {
                        daddr = r.u64(m.off + 8, -2, "layout");
                        dsize = UNDEF;  // implied by dataspace and datatype
                    } else if (lc == 0) {
                        dsize = r.u32(m.off + 8 + 4ull * nd, -2, "layout");
                        compact_off = m.off + 8 + 4ull * nd + 4;
                    } else {
                        throw H5Error{-2, "chunked layout is not supported"};
                    }
                } else {
                    throw H5Error{-2, "layout message version " + std::to_string(v) + " is not supported"};
                }
                have_layout = true;
            } else if (m.type == 0x000B) {
                throw H5Error{-2, "filtered (compressed) datasets are not supported"};
            }
        }
        if (!have_space) throw H5Error{-3, "dataset has no dataspace"};
        if (!have_type) throw H5Error{-4, "dataset has no datatype"};
        if (!have_layout) throw H5Error{-2, "dataset has no layout"};
        uint64_t n = 1;
        for (uint64_t d : dims) {
            if (d && n > (1ull << 40) / d) throw H5Error{-3, "dataspace too large"};
            n *= d;
        }
        const uint64_t bytes = n * (uint64_t)size;
        if (dsize != UNDEF && dsize != bytes) throw H5Error{-3, "stored size does not match the dataspace"};
        data.assign((size_t)n, 0.0);
        uint64_t src = UNDEF;
        if (compact_off != UNDEF) {
            src = compact_off;
        } else if (daddr != UNDEF) {
            src = base + daddr;
        }
        if (src != UNDEF && n) {
            r.need(src, bytes, -3, "dataset data");
            for (uint64_t i = 0; i < n; i++) data[i] = to_double(&r.b[src + i * size], cls, size, be, sgn);
        }
        // An unallocated contiguous dataset reads as the default fill value 0.
        if (type_class) *type_class = cls;
        return 0;
    } catch (const H5Error& e) {
        if (why) *why = e.msg;
        return e.code;
    } catch (const std::bad_alloc&) {
        if (why) *why = "out of host memory";
        return -3;
    }
}

}  // namespace dg
