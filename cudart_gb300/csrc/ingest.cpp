// ingest.cpp -- the reference's scene files read on the host without its
// loaders: Wavefront OBJ with MTL libraries, the camera JSON, PNG textures;
// and PNG output of the resolved image.
//
// What a load produces is what the reference's Scene holds after
// loadObj / loadTextures / loadTriangles (src/geometry/scene.cpp:40-138):
// one record per face in file order (v1 v2 v3, the three shading normals,
// the three uvs, a material id), the material table and the textures'
// linear texels, laid out as crt_scene_desc takes them.
//
// Parsing runs in three parallel passes over line-aligned chunks of the
// file held in memory (count, then v/vt/vn records, then faces written
// straight into the per-face arrays); the few order-dependent lines (o, g,
// usemtl, mtllib) are replayed in file order between the passes.  Numbers
// go through std::from_chars, which rounds correctly like the strtof
// behind the reference's std::stof.
#include "../../include/crt_gb300.h"

#include <algorithm>
#include <atomic>
#include <charconv>
#include <chrono>
#include <fcntl.h>
#include <sys/mman.h>
#include <sys/stat.h>
#include <unistd.h>

#include <cerrno>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <memory>
#include <string>
#include <string_view>
#include <thread>
#include <vector>

namespace crt {
int set_error(int status, const std::string& msg);
const float* stb_texel_table();
}

// Per-face arrays written once, in parallel, by the face pass: left
// uninitialised until then (no serial zero fill).
template <class T>
struct RawArray {
    std::unique_ptr<T[]> p;
    size_t n = 0;
    void allocate(size_t count) {
        p.reset(new T[count]);
        n = count;
    }
    T* data() { return p.get(); }
    const T* data() const { return p.get(); }
    T& operator[](size_t i) { return p[i]; }
};

struct crt_scene_files_s {
    RawArray<float> positions, normals, uvs;      // [n][3][3], [n][3][3], [n][3][2]
    std::vector<uint32_t> material_ids;
    std::vector<crt_material> materials;
    std::vector<uint32_t> texture_dims;
    std::vector<float> texels;
    struct Mesh { std::string name; uint32_t first, count; };
    std::vector<Mesh> meshes;
    crt_scene_files_info info{};
};

namespace {

using crt::set_error;
using Clock = std::chrono::steady_clock;

double ms_since(Clock::time_point t0) {
    return std::chrono::duration<double, std::milli>(Clock::now() - t0).count();
}

template <class F>
void parallel_for(size_t n, F&& f) {
    size_t hw = std::max(1u, std::thread::hardware_concurrency());
    size_t workers = std::min(n, hw);
    if (workers <= 1) {
        for (size_t i = 0; i < n; ++i) f(i);
        return;
    }
    std::atomic<size_t> next{0};
    std::vector<std::thread> pool;
    pool.reserve(workers - 1);
    auto run = [&] {
        for (size_t i; (i = next.fetch_add(1)) < n;) f(i);
    };
    for (size_t w = 1; w < workers; ++w) pool.emplace_back(run);
    run();
    for (auto& t : pool) t.join();
}

bool read_file(const std::string& path, std::string& out, std::string& err) {
    FILE* f = std::fopen(path.c_str(), "rb");
    if (!f) {
        err = "cannot open " + path;
        return false;
    }
    std::fseek(f, 0, SEEK_END);
    long n = std::ftell(f);
    std::fseek(f, 0, SEEK_SET);
    if (n < 0) {
        std::fclose(f);
        err = "cannot read " + path;
        return false;
    }
    out.resize((size_t)n);
    size_t got = n ? std::fread(&out[0], 1, (size_t)n, f) : 0;
    std::fclose(f);
    if (got != (size_t)n) {
        err = "short read of " + path;
        return false;
    }
    return true;
}

// Read-only view of a whole file: a private memory map, so that the parse
// threads fault the pages in parallel instead of one thread copying them.
struct FileView {
    const char* data = "";
    size_t size = 0;
    void* map = nullptr;
    FileView() = default;
    FileView(const FileView&) = delete;
    FileView& operator=(const FileView&) = delete;
    ~FileView() {
        if (map) munmap(map, size);
    }
};

bool map_file(const std::string& path, FileView& fv, std::string& err) {
    const int fd = open(path.c_str(), O_RDONLY);
    if (fd < 0) {
        err = "cannot open " + path;
        return false;
    }
    struct stat st;
    if (fstat(fd, &st) != 0 || !S_ISREG(st.st_mode)) {
        close(fd);
        err = "cannot read " + path;
        return false;
    }
    fv.size = (size_t)st.st_size;
    if (fv.size) {
        void* m = mmap(nullptr, fv.size, PROT_READ, MAP_PRIVATE, fd, 0);
        if (m == MAP_FAILED) {
            close(fd);
            err = "cannot map " + path;
            return false;
        }
        madvise(m, fv.size, MADV_WILLNEED);
        fv.map = m;
        fv.data = static_cast<const char*>(m);
    }
    close(fd);
    return true;
}

bool ends_with(const std::string& s, const char* suffix) {
    size_t k = std::strlen(suffix);
    return s.size() >= k && s.compare(s.size() - k, k, suffix) == 0;
}

// ---------------------------------------------------------------------------
// line and token scanning.  Tokens are separated by runs of spaces and tabs
// (the reference splits on single spaces, so it rejects some files this
// accepts, never the reverse); a trailing '\r' is not part of the line.
// ---------------------------------------------------------------------------
inline bool blank(char c) { return c == ' ' || c == '\t'; }

struct LineText {
    const char* b;      // line start
    const char* e;      // end, without '\n' and a trailing '\r'
    std::string_view head, tail;   // first token; rest with outer blanks trimmed
};

// Splits the line starting at p (buffer end `end`); returns the next line's start.
const char* next_line(const char* p, const char* end, LineText& L) {
    const char* nl = static_cast<const char*>(std::memchr(p, '\n', (size_t)(end - p)));
    const char* le = nl ? nl : end;
    L.b = p;
    L.e = (le > p && le[-1] == '\r') ? le - 1 : le;
    const char* q = p;
    while (q < L.e && blank(*q)) ++q;
    const char* h = q;
    while (q < L.e && !blank(*q)) ++q;
    L.head = std::string_view(h, (size_t)(q - h));
    while (q < L.e && blank(*q)) ++q;
    const char* te = L.e;
    while (te > q && blank(te[-1])) --te;
    L.tail = std::string_view(q, (size_t)(te - q));
    return nl ? nl + 1 : end;
}

// Next blank-separated token of [p, e); empty at the end.
std::string_view next_token(const char*& p, const char* e) {
    while (p < e && blank(*p)) ++p;
    const char* s = p;
    while (p < e && !blank(*p)) ++p;
    return std::string_view(s, (size_t)(p - s));
}

// A number at the start of a token, as std::stof reads it: an optional sign,
// then the longest valid prefix (the rest of the token is ignored).
bool parse_float(std::string_view tok, float& out) {
    const char* p = tok.data();
    const char* e = p + tok.size();
    if (p < e && *p == '+') ++p;
    const char* digits = (p < e && *p == '-') ? p + 1 : p;
    if (e - digits >= 2 && digits[0] == '0' && (digits[1] == 'x' || digits[1] == 'X')) {
        std::string s(tok);   // hexadecimal floats: from_chars wants no prefix
        char* stop = nullptr;
        errno = 0;
        out = std::strtof(s.c_str(), &stop);
        return stop != s.c_str() && errno != ERANGE;
    }
    auto r = std::from_chars(p, e, out, std::chars_format::general);
    return r.ec == std::errc();
}

bool parse_int(std::string_view tok, long long& out) {
    const char* p = tok.data();
    const char* e = p + tok.size();
    if (p < e && *p == '+') ++p;
    auto r = std::from_chars(p, e, out);
    return r.ec == std::errc();
}

// ---------------------------------------------------------------------------
// MTL (objl::Loader::LoadMaterials, src/include/obj_load.h:1015-1186 with
// CudaRT's `type` and `diffuse` keys; defaults of objl::Material,
// obj_load.h:151-161: Ni = 0, type LAMBERT)
// ---------------------------------------------------------------------------
struct MtlMaterial {
    std::string name = "not-initialized";
    float Ka[3] = {0, 0, 0}, Kd[3] = {0, 0, 0}, Ks[3] = {0, 0, 0};
    float Ns = 0.0f, Ni = 0.0f, d = 0.0f, diffuse = 0.0f;
    long long illum = 0;
    std::string type = "LAMBERT";
    std::string map_Kd;
};

int load_mtl(const std::string& path, std::vector<MtlMaterial>& out, uint64_t& bytes) {
    if (!ends_with(path, ".mtl")) return set_error(CRT_ERR_INVALID, "material library is not a .mtl file: " + path);
    std::string text, err;
    if (!read_file(path, text, err)) return set_error(CRT_ERR_INVALID, err);
    bytes += text.size();
    MtlMaterial cur;
    bool listening = false;
    const char* p = text.data();
    const char* end = p + text.size();
    uint64_t line_no = 0;
    auto bad = [&](const char* what) {
        return set_error(CRT_ERR_INVALID, path + ":" + std::to_string(line_no) + ": bad " + what);
    };
    while (p < end) {
        LineText L;
        p = next_line(p, end, L);
        ++line_no;
        const std::string_view h = L.head;
        if (h == "newmtl") {
            if (listening) {
                out.push_back(cur);
                cur = MtlMaterial();
            }
            listening = true;
            // the reference takes the tail only when the raw line has more
            // than 7 characters, else names the material "none"
            cur.name = (L.e - L.b) > 7 ? std::string(L.tail) : std::string("none");
        } else if (h == "Ka" || h == "Kd" || h == "Ks") {
            float* dst = h == "Ka" ? cur.Ka : h == "Kd" ? cur.Kd : cur.Ks;
            const char* q = L.tail.data();
            const char* qe = q + L.tail.size();
            std::string_view t[4];
            int n = 0;
            for (std::string_view tok; n < 4 && !(tok = next_token(q, qe)).empty();) t[n++] = tok;
            if (n != 3) continue;   // the reference skips lines without exactly 3 values
            float v[3];
            for (int k = 0; k < 3; ++k)
                if (!parse_float(t[k], v[k])) return bad("colour");
            std::memcpy(dst, v, sizeof v);
        } else if (h == "Ns" || h == "Ni" || h == "d" || h == "diffuse") {
            float v;
            const char* q = L.tail.data();
            if (!parse_float(next_token(q, q + L.tail.size()), v)) return bad("number");
            (h == "Ns" ? cur.Ns : h == "Ni" ? cur.Ni : h == "d" ? cur.d : cur.diffuse) = v;
        } else if (h == "illum") {
            const char* q = L.tail.data();
            if (!parse_int(next_token(q, q + L.tail.size()), cur.illum)) return bad("illum");
        } else if (h == "map_Kd") {
            cur.map_Kd = std::string(L.tail);
        } else if (h == "type") {
            cur.type = std::string(L.tail);
        }
    }
    out.push_back(cur);   // the last material, even without a newmtl line
    return CRT_OK;
}

// ---------------------------------------------------------------------------
// material table.  materialFromMtl (scene.cpp:175-190): ka = Ka * 3, bsdf
// from `type`.  The reference merges materials through a std::map ordered by
// materialComparator (material.h:57-79) and then gives each mesh the first
// table entry that compares equal under Material::operator== (material.h:
// 31-54), whose float3 `!=` is true only when all three components differ
// (linalg.h:12).  Both steps are restated here so that the same files give
// the same table; CRT_LOAD_EXACT_MATERIALS gives each MTL material its own
// entry instead.
// ---------------------------------------------------------------------------
struct TableMaterial {
    int32_t bsdf;
    float kd[3], ka3[3], ks[3];
    float ns, ni, diffuse;
    float Ka[3];          // the MTL value (the scene applies the 3x gain itself)
    int32_t texture;
};

int32_t bsdf_of(const std::string& type) {
    static const std::pair<const char*, int32_t> names[] = {
        {"LAMBERT", CRT_BSDF_DIFFUSE},   {"SPECULAR", CRT_BSDF_SPECULAR},
        {"DIFFSPEC", CRT_BSDF_DIFFSPEC}, {"MICROFACET", CRT_BSDF_MICROFACET},
        {"REFRACTIVE", CRT_BSDF_REFRACTIVE}, {"EMISSIVE", CRT_BSDF_EMISSIVE}};
    for (const auto& n : names)
        if (type == n.first) return n.second;
    return CRT_BSDF_DIFFUSE;
}

TableMaterial table_material(const MtlMaterial& m) {
    TableMaterial t;
    t.bsdf = bsdf_of(m.type);
    for (int k = 0; k < 3; ++k) {
        t.kd[k] = m.Kd[k];
        t.ka3[k] = m.Ka[k] * 3.0f;
        t.ks[k] = m.Ks[k];
        t.Ka[k] = m.Ka[k];
    }
    t.ns = m.Ns;
    t.ni = m.Ni;
    t.diffuse = m.diffuse;
    t.texture = CRT_NO_TEXTURE;
    return t;
}

bool any_below(const float* a, const float* b) { return a[0] < b[0] || a[1] < b[1] || a[2] < b[2]; }
bool all_differ(const float* a, const float* b) { return a[0] != b[0] && a[1] != b[1] && a[2] != b[2]; }

// The reference's map order: not a strict weak order, so which materials
// merge depends on the tree's insertion history, as in the reference.
struct ReferenceOrder {
    bool operator()(const TableMaterial& a, const TableMaterial& b) const {
        if (a.bsdf != b.bsdf) return a.bsdf < b.bsdf;
        if (any_below(a.kd, b.kd)) return true;
        if (any_below(a.ka3, b.ka3)) return true;
        if (any_below(a.ks, b.ks)) return true;
        if (a.ns < b.ns) return true;
        return a.ni < b.ni;
    }
};

bool reference_equal(const TableMaterial& a, const TableMaterial& b) {
    return a.bsdf == b.bsdf && !all_differ(a.kd, b.kd) && !all_differ(a.ka3, b.ka3) &&
           !all_differ(a.ks, b.ks) && a.ns == b.ns && a.ni == b.ni && a.diffuse == b.diffuse;
}

crt_material to_abi(const TableMaterial& t) {
    crt_material m;
    m.bsdf = t.bsdf;
    m.texture = t.texture;
    for (int k = 0; k < 3; ++k) {
        m.kd[k] = t.kd[k];
        m.ka[k] = t.Ka[k];
        m.ks[k] = t.ks[k];
    }
    m.ns = t.ns;
    m.ni = t.ni;
    m.diffuse = t.diffuse;
    return m;
}

// ---------------------------------------------------------------------------
// OBJ (objl::Loader::LoadFile, obj_load.h:441-720; faces as
// GenVerticesFromRawOBJ, :730-844)
// ---------------------------------------------------------------------------
enum LineKind : uint8_t { L_OTHER, L_V, L_VT, L_VN, L_F, L_GROUP, L_USEMTL, L_MTLLIB };

LineKind classify(const LineText& L) {
    const std::string_view h = L.head;
    // the reference opens a group on `o`, `g`, or any line whose first
    // character is 'g'
    if (h == "o" || h == "g" || (L.b < L.e && *L.b == 'g')) return L_GROUP;
    if (h == "v") return L_V;
    if (h == "vt") return L_VT;
    if (h == "vn") return L_VN;
    if (h == "f") return L_F;
    if (h == "usemtl") return L_USEMTL;
    if (h == "mtllib") return L_MTLLIB;
    return L_OTHER;
}

struct Event {
    LineKind kind;
    bool named;           // `o` or `g` (else a line that only starts with 'g')
    uint64_t tri;         // faces' triangles before the line (chunk-local)
    std::string text;
};

struct Chunk {
    const char* b;
    const char* e;
    uint64_t lines = 0, nv = 0, nvt = 0, nvn = 0, ntri = 0, npoly = 0;
    uint64_t line0 = 0, v0 = 0, vt0 = 0, vn0 = 0, tri0 = 0;
    std::vector<Event> events;
    uint64_t err_line = 0;     // 1-based line of the first error in the chunk
    std::string err;
    void fail(uint64_t local_line, const std::string& what) {
        if (err.empty()) {
            err_line = line0 + local_line;
            err = what;
        }
    }
};

int count_face_vertices(std::string_view tail) {
    const char* p = tail.data();
    const char* e = p + tail.size();
    int n = 0;
    while (!next_token(p, e).empty()) ++n;
    return n;
}

// One face vertex "p", "p/t", "p//n" or "p/t/n"; a single trailing '/' is
// ignored, as the reference's split drops it.  Indices are 1-based, or
// negative counting back from the records read so far.
struct FaceVertex { int64_t p, t, n; };   // -1: absent

bool resolve(std::string_view s, uint64_t count, int64_t& out) {
    long long v;
    if (s.empty() || !parse_int(s, v)) return false;
    long long idx = v < 0 ? (long long)count + v : v - 1;
    if (idx < 0 || (unsigned long long)idx >= count) return false;
    out = idx;
    return true;
}

bool parse_face_vertex(std::string_view tok, uint64_t nv, uint64_t nvt, uint64_t nvn, FaceVertex& fv) {
    std::string_view part[4];
    int n = 0;
    size_t s = 0;
    while (n < 4) {
        size_t slash = tok.find('/', s);
        part[n++] = tok.substr(s, slash == std::string_view::npos ? std::string_view::npos : slash - s);
        if (slash == std::string_view::npos) break;
        s = slash + 1;
    }
    if (n > 1 && part[n - 1].empty()) --n;      // "p/" or "p/t/"
    fv.t = fv.n = -1;
    if (n < 1 || n > 3 || !resolve(part[0], nv, fv.p)) return false;
    if (n >= 2 && !part[1].empty() && !resolve(part[1], nvt, fv.t)) return false;
    if (n == 2 && part[1].empty()) return false;
    if (n == 3 && !resolve(part[2], nvn, fv.n)) return false;
    return true;
}

}  // namespace

// ---------------------------------------------------------------------------
// PNG decoding (own inflate, RFC 1950/1951; PNG filters and Adam7, ISO/IEC
// 15948) into the texels stbi_loadf returns for 8-bit data:
// (float)pow(b / 255, 2.2) per colour channel (stb_image's LDR-to-HDR
// conversion with its default gamma); 16-bit samples keep their high byte,
// as stbi_loadf converts them to 8 bits first.
// ---------------------------------------------------------------------------
namespace {

struct BitReader {
    const uint8_t* p;
    const uint8_t* e;
    uint64_t buf = 0;
    int bits = 0;          // bits held in buf
    uint64_t padded = 0;   // zero bytes fed after the end of the input
    void refill() {
        while (bits <= 56) {
            uint64_t byte = 0;
            if (p < e) byte = *p++;
            else ++padded;
            buf |= byte << bits;
            bits += 8;
        }
    }
    uint32_t peek(int n) {
        if (bits < n) refill();
        return (uint32_t)(buf & ((1ull << n) - 1));
    }
    void drop(int n) {
        buf >>= n;
        bits -= n;
    }
    uint32_t take(int n) {
        if (n == 0) return 0;
        uint32_t v = peek(n);
        drop(n);
        return v;
    }
    // some of the zero padding was consumed: the stream is truncated
    bool truncated() const { return padded * 8 > (uint64_t)bits; }
};

// Canonical Huffman code with a 9-bit first-level table.
struct Huffman {
    static constexpr int kFast = 9;
    uint16_t fast[1 << kFast];       // (length << 12) | symbol, 0 = slow path
    uint16_t count[16];
    uint16_t symbol[320];
    bool build(const uint8_t* lengths, int n) {
        std::memset(count, 0, sizeof count);
        std::memset(fast, 0, sizeof fast);
        for (int i = 0; i < n; ++i) count[lengths[i]]++;
        count[0] = 0;
        int left = 1;
        for (int len = 1; len < 16; ++len) {
            left = (left << 1) - count[len];
            if (left < 0) return false;   // over-subscribed
        }
        uint16_t offs[16];
        offs[1] = 0;
        for (int len = 1; len < 15; ++len) offs[len + 1] = offs[len] + count[len];
        for (int i = 0; i < n; ++i)
            if (lengths[i]) symbol[offs[lengths[i]]++] = (uint16_t)i;
        // first-level table: codes of <= kFast bits, stored bit-reversed
        int code = 0, idx = 0;
        for (int len = 1; len <= kFast; ++len) {
            for (int k = 0; k < count[len]; ++k, ++code, ++idx) {
                int rev = 0;
                for (int b = 0; b < len; ++b) rev |= ((code >> b) & 1) << (len - 1 - b);
                for (int fill = rev; fill < (1 << kFast); fill += 1 << len)
                    fast[fill] = (uint16_t)((len << 12) | symbol[idx]);
            }
            code <<= 1;
        }
        return true;
    }
    int decode(BitReader& br) const {
        uint32_t bitsv = br.peek(15);
        uint16_t f = fast[bitsv & ((1 << kFast) - 1)];
        if (f) {
            br.drop(f >> 12);
            return f & 0xFFF;
        }
        // slow path: walk the canonical code one bit at a time
        int code = 0, first = 0, index = 0;
        for (int len = 1; len < 16; ++len) {
            code |= (bitsv >> (len - 1)) & 1;
            int c = count[len];
            if (code - c < first) {
                br.drop(len);
                return symbol[index + (code - first)];
            }
            index += c;
            first = (first + c) << 1;
            code <<= 1;
        }
        return -1;
    }
};

const uint16_t kLenBase[29] = {3, 4, 5, 6, 7, 8, 9, 10, 11, 13, 15, 17, 19, 23, 27,
                               31, 35, 43, 51, 59, 67, 83, 99, 115, 131, 163, 195, 227, 258};
const uint8_t kLenExtra[29] = {0, 0, 0, 0, 0, 0, 0, 0, 1, 1, 1, 1, 2, 2, 2,
                               2, 3, 3, 3, 3, 4, 4, 4, 4, 5, 5, 5, 5, 0};
const uint16_t kDistBase[30] = {1, 2, 3, 4, 5, 7, 9, 13, 17, 25, 33, 49, 65, 97, 129,
                                193, 257, 385, 513, 769, 1025, 1537, 2049, 3073, 4097,
                                6145, 8193, 12289, 16385, 24577};
const uint8_t kDistExtra[30] = {0, 0, 0, 0, 1, 1, 2, 2, 3, 3, 4, 4, 5, 5, 6,
                                6, 7, 7, 8, 8, 9, 9, 10, 10, 11, 11, 12, 12, 13, 13};

// zlib stream -> out (exactly `expect` bytes are wanted; more is an error).
bool inflate_zlib(const uint8_t* src, size_t n, std::vector<uint8_t>& out, size_t expect, std::string& err) {
    if (n < 2) { err = "zlib stream too short"; return false; }
    const unsigned cmf = src[0], flg = src[1];
    if ((cmf & 15) != 8 || (cmf >> 4) > 7 || ((cmf << 8) | flg) % 31 != 0 || (flg & 32)) {
        err = "bad zlib header";
        return false;
    }
    out.clear();
    out.reserve(expect);
    BitReader br{src + 2, src + n};
    Huffman lit, dist;
    bool last = false;
    while (!last) {
        last = br.take(1);
        const uint32_t type = br.take(2);
        if (type == 0) {
            br.drop(br.bits & 7);   // to a byte boundary
            const uint32_t len = br.take(16), nlen = br.take(16);
            if ((len ^ 0xFFFF) != nlen) { err = "bad stored block"; return false; }
            for (uint32_t i = 0; i < len; ++i) out.push_back((uint8_t)br.take(8));
        } else if (type == 1 || type == 2) {
            uint8_t lengths[320];
            int nlit = 288, ndist = 32;
            if (type == 1) {
                for (int i = 0; i < 144; ++i) lengths[i] = 8;
                for (int i = 144; i < 256; ++i) lengths[i] = 9;
                for (int i = 256; i < 280; ++i) lengths[i] = 7;
                for (int i = 280; i < 288; ++i) lengths[i] = 8;
                for (int i = 0; i < 32; ++i) lengths[288 + i] = 5;
            } else {
                nlit = (int)br.take(5) + 257;
                ndist = (int)br.take(5) + 1;
                const int ncode = (int)br.take(4) + 4;
                static const uint8_t order[19] = {16, 17, 18, 0, 8, 7, 9, 6, 10, 5,
                                                  11, 4, 12, 3, 13, 2, 14, 1, 15};
                uint8_t cl[19] = {0};
                for (int i = 0; i < ncode; ++i) cl[order[i]] = (uint8_t)br.take(3);
                Huffman clh;
                if (!clh.build(cl, 19)) { err = "bad code-length code"; return false; }
                int i = 0;
                while (i < nlit + ndist) {
                    int sym = clh.decode(br);
                    if (sym < 0) { err = "bad code length"; return false; }
                    if (sym < 16) {
                        lengths[i++] = (uint8_t)sym;
                        continue;
                    }
                    int rep;
                    uint8_t v = 0;
                    if (sym == 16) {
                        if (i == 0) { err = "repeat with no previous length"; return false; }
                        v = lengths[i - 1];
                        rep = 3 + (int)br.take(2);
                    } else if (sym == 17) {
                        rep = 3 + (int)br.take(3);
                    } else {
                        rep = 11 + (int)br.take(7);
                    }
                    if (i + rep > nlit + ndist) { err = "code lengths overflow"; return false; }
                    while (rep--) lengths[i++] = v;
                }
                if (lengths[256] == 0) { err = "no end-of-block code"; return false; }
                // the distance lengths start right after the literal lengths
                std::memmove(lengths + 288, lengths + nlit, (size_t)ndist);
                for (int k = nlit; k < 288; ++k) lengths[k] = 0;
                for (int k = ndist; k < 32; ++k) lengths[288 + k] = 0;
            }
            if (!lit.build(lengths, 288) || !dist.build(lengths + 288, 32)) {
                err = "bad Huffman code";
                return false;
            }
            for (;;) {
                int sym = lit.decode(br);
                if (sym < 0 || br.truncated()) { err = "bad literal/length code"; return false; }
                if (sym < 256) {
                    out.push_back((uint8_t)sym);
                } else if (sym == 256) {
                    break;
                } else {
                    sym -= 257;
                    if (sym >= 29) { err = "bad length symbol"; return false; }
                    const uint32_t len = kLenBase[sym] + br.take(kLenExtra[sym]);
                    int ds = dist.decode(br);
                    if (ds < 0 || ds >= 30) { err = "bad distance code"; return false; }
                    const uint32_t d = kDistBase[ds] + br.take(kDistExtra[ds]);
                    if (d > out.size()) { err = "distance beyond the output"; return false; }
                    size_t from = out.size() - d;
                    for (uint32_t k = 0; k < len; ++k) out.push_back(out[from + k]);
                }
                if (out.size() > expect) { err = "more image data than the header allows"; return false; }
            }
        } else {
            err = "bad block type";
            return false;
        }
        if (br.truncated()) { err = "truncated zlib stream"; return false; }
        if (out.size() > expect) { err = "more image data than the header allows"; return false; }
    }
    return true;
}

inline uint8_t paeth(int a, int b, int c) {
    int p = a + b - c;
    int pa = std::abs(p - a), pb = std::abs(p - b), pc = std::abs(p - c);
    if (pa <= pb && pa <= pc) return (uint8_t)a;
    if (pb <= pc) return (uint8_t)b;
    return (uint8_t)c;
}

// Undo the filters of one (sub)image in place; rows of `stride` bytes, each
// preceded by its filter byte.
bool unfilter(uint8_t* data, uint32_t rows, size_t stride, int bpp, std::vector<uint8_t>& img,
              std::string& err) {
    img.assign((size_t)rows * stride, 0);
    for (uint32_t y = 0; y < rows; ++y) {
        const uint8_t ft = data[y * (stride + 1)];
        const uint8_t* in = data + y * (stride + 1) + 1;
        uint8_t* cur = img.data() + (size_t)y * stride;
        const uint8_t* up = y ? cur - stride : nullptr;
        for (size_t i = 0; i < stride; ++i) {
            const int a = i >= (size_t)bpp ? cur[i - bpp] : 0;
            const int b = up ? up[i] : 0;
            const int c = (up && i >= (size_t)bpp) ? up[i - bpp] : 0;
            int v;
            switch (ft) {
                case 0: v = in[i]; break;
                case 1: v = in[i] + a; break;
                case 2: v = in[i] + b; break;
                case 3: v = in[i] + ((a + b) >> 1); break;
                case 4: v = in[i] + paeth(a, b, c); break;
                default: err = "bad filter type " + std::to_string(ft); return false;
            }
            cur[i] = (uint8_t)v;
        }
    }
    return true;
}

uint32_t be32(const uint8_t* p) {
    return ((uint32_t)p[0] << 24) | ((uint32_t)p[1] << 16) | ((uint32_t)p[2] << 8) | p[3];
}

const float* gamma_lut() {
    static const std::vector<float> lut = [] {
        std::vector<float> t(256);
        for (int b = 0; b < 256; ++b) t[b] = (float)std::pow((double)((float)b / 255.0f), (double)2.2f);
        return t;
    }();
    return lut.data();
}

}  // namespace

// The same table for crt_scene_create's RGBA8 texels.
const float* crt::stb_texel_table() { return gamma_lut(); }

namespace {

// Decodes a PNG file into rgb texels (8-bit sample values per channel).
struct Png {
    uint32_t w = 0, h = 0;
    std::vector<uint8_t> rgb;   // [h*w][3]
};

bool decode_png(const std::string& bytes, Png& img, std::string& err) {
    const uint8_t* s = reinterpret_cast<const uint8_t*>(bytes.data());
    const size_t n = bytes.size();
    static const uint8_t sig[8] = {0x89, 'P', 'N', 'G', '\r', '\n', 0x1A, '\n'};
    if (n < 8 || std::memcmp(s, sig, 8) != 0) { err = "not a PNG file"; return false; }
    size_t pos = 8;
    uint32_t w = 0, h = 0;
    int depth = 0, ctype = -1, interlace = 0;
    std::vector<uint8_t> idat, palette;
    bool seen_ihdr = false, seen_iend = false;
    while (pos + 12 <= n && !seen_iend) {
        const uint32_t len = be32(s + pos);
        const uint8_t* type = s + pos + 4;
        const uint8_t* data = s + pos + 8;
        if (len > n - pos - 12) { err = "truncated PNG chunk"; return false; }
        const std::string t(reinterpret_cast<const char*>(type), 4);
        if (t == "IHDR") {
            if (len != 13 || seen_ihdr) { err = "bad IHDR"; return false; }
            w = be32(data);
            h = be32(data + 4);
            depth = data[8];
            ctype = data[9];
            interlace = data[12];
            if (data[10] != 0 || data[11] != 0 || interlace > 1) { err = "unsupported PNG compression/filter/interlace"; return false; }
            seen_ihdr = true;
        } else if (!seen_ihdr) {
            err = "PNG chunk before IHDR";
            return false;
        } else if (t == "PLTE") {
            if (len % 3 || len > 768) { err = "bad PLTE"; return false; }
            palette.assign(data, data + len);
        } else if (t == "IDAT") {
            idat.insert(idat.end(), data, data + len);
        } else if (t == "IEND") {
            seen_iend = true;
        } else if (!(type[0] & 0x20)) {
            err = "unsupported critical PNG chunk " + t;
            return false;
        }
        pos += 12 + (size_t)len;   // CRCs are not checked (nor does stb_image)
    }
    if (!seen_ihdr || idat.empty()) { err = "PNG without IHDR or IDAT"; return false; }
    if (w == 0 || h == 0 || w > (1u << 24) || h > (1u << 24)) { err = "bad PNG size"; return false; }
    int channels;
    switch (ctype) {
        case 0: channels = 1; if (depth != 1 && depth != 2 && depth != 4 && depth != 8 && depth != 16) ctype = -2; break;
        case 2: channels = 3; if (depth != 8 && depth != 16) ctype = -2; break;
        case 3: channels = 1; if (depth != 1 && depth != 2 && depth != 4 && depth != 8) ctype = -2; break;
        case 4: channels = 2; if (depth != 8 && depth != 16) ctype = -2; break;
        case 6: channels = 4; if (depth != 8 && depth != 16) ctype = -2; break;
        default: err = "bad PNG colour type"; return false;
    }
    if (ctype == -2) { err = "bad PNG bit depth"; return false; }
    if (ctype == 3 && palette.empty()) { err = "palette image without PLTE"; return false; }
    const int bits_pp = channels * depth;
    const int bpp = std::max(1, bits_pp / 8);
    struct Pass { uint32_t x0, y0, dx, dy; };
    static const Pass adam7[7] = {{0, 0, 8, 8}, {4, 0, 8, 8}, {0, 4, 4, 8}, {2, 0, 4, 4},
                                  {0, 2, 2, 4}, {1, 0, 2, 2}, {0, 1, 1, 2}};
    static const Pass whole[1] = {{0, 0, 1, 1}};
    const Pass* passes = interlace ? adam7 : whole;
    const int npass = interlace ? 7 : 1;
    size_t expect = 0;
    for (int k = 0; k < npass; ++k) {
        const uint64_t pw = (w - passes[k].x0 + passes[k].dx - 1) / passes[k].dx;
        const uint64_t ph = (h - passes[k].y0 + passes[k].dy - 1) / passes[k].dy;
        if (pw && ph) expect += (size_t)ph * (1 + (size_t)((pw * bits_pp + 7) / 8));
    }
    std::vector<uint8_t> raw;
    if (!inflate_zlib(idat.data(), idat.size(), raw, expect, err)) return false;
    if (raw.size() != expect) { err = "PNG image data has the wrong size"; return false; }
    img.w = w;
    img.h = h;
    img.rgb.assign((size_t)w * h * 3, 0);
    size_t off = 0;
    std::vector<uint8_t> rows;
    for (int k = 0; k < npass; ++k) {
        const Pass& P = passes[k];
        const uint32_t pw = (uint32_t)((w - P.x0 + P.dx - 1) / P.dx);
        const uint32_t ph = (uint32_t)((h - P.y0 + P.dy - 1) / P.dy);
        if (!pw || !ph) continue;
        const size_t stride = ((size_t)pw * bits_pp + 7) / 8;
        if (!unfilter(raw.data() + off, ph, stride, bpp, rows, err)) return false;
        off += (size_t)ph * (stride + 1);
        for (uint32_t y = 0; y < ph; ++y) {
            const uint8_t* r = rows.data() + (size_t)y * stride;
            for (uint32_t x = 0; x < pw; ++x) {
                uint8_t c[4];
                for (int ch = 0; ch < channels; ++ch) {
                    const size_t sample = (size_t)x * channels + ch;
                    uint32_t v;
                    if (depth == 16) {
                        v = r[2 * sample];   // high byte
                    } else if (depth == 8) {
                        v = r[sample];
                    } else {
                        const size_t bit = sample * depth;
                        v = (r[bit >> 3] >> (8 - depth - (bit & 7))) & ((1u << depth) - 1);
                        if (ctype == 0) v = v * (255u / ((1u << depth) - 1));
                    }
                    c[ch] = (uint8_t)v;
                }
                uint8_t* o = img.rgb.data() + ((size_t)(P.y0 + y * P.dy) * w + P.x0 + x * P.dx) * 3;
                if (ctype == 3) {
                    if ((size_t)c[0] * 3 + 2 >= palette.size()) { err = "palette index out of range"; return false; }
                    o[0] = palette[c[0] * 3];
                    o[1] = palette[c[0] * 3 + 1];
                    o[2] = palette[c[0] * 3 + 2];
                } else if (channels <= 2) {
                    // grey (and grey + alpha): the reference reads three
                    // consecutive floats of a one- or two-channel image;
                    // the grey value is replicated here instead
                    o[0] = o[1] = o[2] = c[0];
                } else {
                    o[0] = c[0];
                    o[1] = c[1];
                    o[2] = c[2];
                }
            }
        }
    }
    return true;
}

// ---------------------------------------------------------------------------
// PNG encoding: per-row filter by the minimum sum of absolute differences,
// deflate with a greedy hash-chain LZ77 and the fixed Huffman code.
// ---------------------------------------------------------------------------
struct BitWriter {
    std::vector<uint8_t>& out;
    uint64_t buf = 0;
    int bits = 0;
    explicit BitWriter(std::vector<uint8_t>& o) : out(o) {}
    void put(uint32_t v, int n) {   // n <= 32, LSB first
        buf |= (uint64_t)v << bits;
        bits += n;
        while (bits >= 8) {
            out.push_back((uint8_t)buf);
            buf >>= 8;
            bits -= 8;
        }
    }
    void put_rev(uint32_t code, int n) {   // Huffman codes go MSB first
        uint32_t r = 0;
        for (int i = 0; i < n; ++i) r |= ((code >> i) & 1) << (n - 1 - i);
        put(r, n);
    }
    void flush() {
        if (bits) out.push_back((uint8_t)buf);
        buf = 0;
        bits = 0;
    }
};

void fixed_literal(BitWriter& bw, int sym) {
    if (sym < 144) bw.put_rev(0x30 + sym, 8);
    else if (sym < 256) bw.put_rev(0x190 + sym - 144, 9);
    else if (sym < 280) bw.put_rev(sym - 256, 7);
    else bw.put_rev(0xC0 + sym - 280, 8);
}

void deflate_fixed(const std::vector<uint8_t>& in, std::vector<uint8_t>& out) {
    BitWriter bw(out);
    bw.put(1, 1);   // final block
    bw.put(1, 2);   // fixed Huffman
    const size_t n = in.size();
    constexpr int kHashBits = 15;
    constexpr size_t kWindow = 32768;
    std::vector<int32_t> head(1 << kHashBits, -1), prev(n, -1);
    auto hash = [&](size_t i) {
        return ((uint32_t)in[i] * 506832829u ^ (uint32_t)in[i + 1] * 2654435761u ^ (uint32_t)in[i + 2]) &
               ((1u << kHashBits) - 1);
    };
    size_t i = 0;
    while (i < n) {
        int best_len = 0;
        size_t best_d = 0;
        if (i + 3 <= n) {
            const uint32_t hv = hash(i);
            int64_t cand = head[hv];   // < 2^31: the caller bounds the image size
            for (int chain = 0; cand >= 0 && chain < 32; ++chain, cand = prev[cand]) {
                const size_t d = i - (size_t)cand;
                if (d > kWindow) break;
                int len = 0;
                const int max_len = (int)std::min<size_t>(258, n - i);
                while (len < max_len && in[cand + len] == in[i + len]) ++len;
                if (len > best_len) {
                    best_len = len;
                    best_d = d;
                    if (len == max_len) break;
                }
            }
        }
        const size_t step = best_len >= 3 ? (size_t)best_len : 1;
        for (size_t k = 0; k < step; ++k) {   // insert every covered position
            if (i + k + 3 <= n) {
                const uint32_t hv = hash(i + k);
                prev[i + k] = head[hv];
                head[hv] = (int32_t)(i + k);
            }
        }
        if (best_len >= 3) {
            int ls = 28;
            while (kLenBase[ls] > best_len) --ls;
            fixed_literal(bw, 257 + ls);
            bw.put((uint32_t)(best_len - kLenBase[ls]), kLenExtra[ls]);
            int ds = 29;
            while (kDistBase[ds] > best_d) --ds;
            bw.put_rev((uint32_t)ds, 5);
            bw.put((uint32_t)(best_d - kDistBase[ds]), kDistExtra[ds]);
        } else {
            fixed_literal(bw, in[i]);
        }
        i += step;
    }
    fixed_literal(bw, 256);
    bw.flush();
}

uint32_t crc32_of(const uint8_t* p, size_t n, uint32_t crc = 0) {
    static const std::vector<uint32_t> table = [] {
        std::vector<uint32_t> t(256);
        for (uint32_t k = 0; k < 256; ++k) {
            uint32_t c = k;
            for (int b = 0; b < 8; ++b) c = (c & 1) ? 0xEDB88320u ^ (c >> 1) : c >> 1;
            t[k] = c;
        }
        return t;
    }();
    crc = ~crc;
    for (size_t i = 0; i < n; ++i) crc = table[(crc ^ p[i]) & 0xFF] ^ (crc >> 8);
    return ~crc;
}

void put_be32(std::vector<uint8_t>& o, uint32_t v) {
    o.push_back((uint8_t)(v >> 24));
    o.push_back((uint8_t)(v >> 16));
    o.push_back((uint8_t)(v >> 8));
    o.push_back((uint8_t)v);
}

void put_chunk(std::vector<uint8_t>& o, const char* type, const std::vector<uint8_t>& data) {
    put_be32(o, (uint32_t)data.size());
    const size_t start = o.size();
    o.insert(o.end(), type, type + 4);
    o.insert(o.end(), data.begin(), data.end());
    put_be32(o, crc32_of(o.data() + start, o.size() - start));
}

std::vector<uint8_t> encode_png(uint32_t w, uint32_t h, const uint8_t* rgba) {
    const size_t stride = (size_t)w * 4;
    std::vector<uint8_t> filtered;
    filtered.reserve((stride + 1) * h);
    std::vector<uint8_t> cand(stride);
    for (uint32_t y = 0; y < h; ++y) {
        const uint8_t* cur = rgba + y * stride;
        const uint8_t* up = y ? cur - stride : nullptr;
        int best_f = 0;
        uint64_t best_cost = UINT64_MAX;
        for (int f = 0; f < 5; ++f) {
            uint64_t cost = 0;
            for (size_t i = 0; i < stride; ++i) {
                const int a = i >= 4 ? cur[i - 4] : 0, b = up ? up[i] : 0,
                          c = (up && i >= 4) ? up[i - 4] : 0;
                const int pred = f == 0 ? 0 : f == 1 ? a : f == 2 ? b : f == 3 ? (a + b) >> 1 : paeth(a, b, c);
                cost += (uint64_t)std::abs((int)(int8_t)(uint8_t)(cur[i] - pred));
            }
            if (cost < best_cost) {
                best_cost = cost;
                best_f = f;
            }
        }
        filtered.push_back((uint8_t)best_f);
        for (size_t i = 0; i < stride; ++i) {
            const int a = i >= 4 ? cur[i - 4] : 0, b = up ? up[i] : 0, c = (up && i >= 4) ? up[i - 4] : 0;
            const int pred = best_f == 0 ? 0 : best_f == 1 ? a : best_f == 2 ? b : best_f == 3 ? (a + b) >> 1 : paeth(a, b, c);
            cand[i] = (uint8_t)(cur[i] - pred);
        }
        filtered.insert(filtered.end(), cand.begin(), cand.end());
    }
    std::vector<uint8_t> z = {0x78, 0x01};
    deflate_fixed(filtered, z);
    uint32_t s1 = 1, s2 = 0;   // Adler-32
    for (uint8_t b : filtered) {
        s1 = (s1 + b) % 65521;
        s2 = (s2 + s1) % 65521;
    }
    put_be32(z, (s2 << 16) | s1);
    std::vector<uint8_t> png = {0x89, 'P', 'N', 'G', '\r', '\n', 0x1A, '\n'};
    std::vector<uint8_t> ihdr;
    put_be32(ihdr, w);
    put_be32(ihdr, h);
    ihdr.insert(ihdr.end(), {8, 6, 0, 0, 0});
    put_chunk(png, "IHDR", ihdr);
    put_chunk(png, "IDAT", z);
    put_chunk(png, "IEND", {});
    return png;
}

// ---------------------------------------------------------------------------
// JSON (the subset picojson parses for the camera file): numbers as strtod
// reads the characters [0-9+-.eE], strings with the standard escapes.
// ---------------------------------------------------------------------------
struct Json {
    enum Type { NUL, BOOL, NUM, STR, ARR, OBJ } type = NUL;
    double num = 0;
    bool b = false;
    std::string str;
    std::vector<Json> arr;
    std::vector<std::pair<std::string, Json>> obj;
    const Json* get(const std::string& key) const {
        const Json* found = nullptr;
        for (const auto& kv : obj)
            if (kv.first == key) found = &kv.second;   // the last duplicate wins
        return found;
    }
};

struct JsonParser {
    const char* p;
    const char* e;
    std::string err;
    int depth = 0;
    JsonParser(const char* b, const char* end) : p(b), e(end) {}
    void ws() {
        while (p < e && (*p == ' ' || *p == '\t' || *p == '\n' || *p == '\r')) ++p;
    }
    bool fail(const char* what) {
        if (err.empty()) err = what;
        return false;
    }
    bool literal(const char* word) {
        size_t k = std::strlen(word);
        if ((size_t)(e - p) < k || std::memcmp(p, word, k) != 0) return fail("bad literal");
        p += k;
        return true;
    }
    bool string(std::string& out) {
        if (p >= e || *p != '"') return fail("expected a string");
        ++p;
        out.clear();
        while (p < e && *p != '"') {
            char c = *p++;
            if (c != '\\') {
                out.push_back(c);
                continue;
            }
            if (p >= e) return fail("bad escape");
            c = *p++;
            switch (c) {
                case '"': case '\\': case '/': out.push_back(c); break;
                case 'b': out.push_back('\b'); break;
                case 'f': out.push_back('\f'); break;
                case 'n': out.push_back('\n'); break;
                case 'r': out.push_back('\r'); break;
                case 't': out.push_back('\t'); break;
                case 'u': {
                    if (e - p < 4) return fail("bad \\u escape");
                    unsigned v = 0;
                    for (int k = 0; k < 4; ++k) {
                        char h = *p++;
                        v <<= 4;
                        if (h >= '0' && h <= '9') v |= (unsigned)(h - '0');
                        else if (h >= 'a' && h <= 'f') v |= (unsigned)(h - 'a' + 10);
                        else if (h >= 'A' && h <= 'F') v |= (unsigned)(h - 'A' + 10);
                        else return fail("bad \\u escape");
                    }
                    // UTF-8 of the code unit (surrogate pairs are not joined;
                    // the camera file's keys are ASCII)
                    if (v < 0x80) out.push_back((char)v);
                    else if (v < 0x800) { out.push_back((char)(0xC0 | (v >> 6))); out.push_back((char)(0x80 | (v & 63))); }
                    else { out.push_back((char)(0xE0 | (v >> 12))); out.push_back((char)(0x80 | ((v >> 6) & 63))); out.push_back((char)(0x80 | (v & 63))); }
                    break;
                }
                default: return fail("bad escape");
            }
        }
        if (p >= e) return fail("unterminated string");
        ++p;
        return true;
    }
    bool value(Json& v) {
        if (++depth > 64) return fail("JSON nested too deeply");
        ws();
        if (p >= e) return fail("unexpected end of JSON");
        bool ok = true;
        if (*p == '{') {
            v.type = Json::OBJ;
            ++p;
            ws();
            if (p < e && *p == '}') {
                ++p;
            } else {
                for (;;) {
                    ws();
                    std::string key;
                    Json item;
                    if (!string(key)) return false;
                    ws();
                    if (p >= e || *p != ':') return fail("expected ':'");
                    ++p;
                    if (!value(item)) return false;
                    v.obj.emplace_back(std::move(key), std::move(item));
                    ws();
                    if (p < e && *p == ',') { ++p; continue; }
                    if (p < e && *p == '}') { ++p; break; }
                    return fail("expected ',' or '}'");
                }
            }
        } else if (*p == '[') {
            v.type = Json::ARR;
            ++p;
            ws();
            if (p < e && *p == ']') {
                ++p;
            } else {
                for (;;) {
                    Json item;
                    if (!value(item)) return false;
                    v.arr.push_back(std::move(item));
                    ws();
                    if (p < e && *p == ',') { ++p; continue; }
                    if (p < e && *p == ']') { ++p; break; }
                    return fail("expected ',' or ']'");
                }
            }
        } else if (*p == '"') {
            v.type = Json::STR;
            ok = string(v.str);
        } else if (*p == 't') {
            v.type = Json::BOOL;
            v.b = true;
            ok = literal("true");
        } else if (*p == 'f') {
            v.type = Json::BOOL;
            ok = literal("false");
        } else if (*p == 'n') {
            ok = literal("null");
        } else {
            const char* s = p;
            while (p < e && (std::strchr("0123456789+-.eE", *p) != nullptr) && *p) ++p;
            if (p == s) return fail("unexpected character in JSON");
            std::string digits(s, (size_t)(p - s));
            char* stop = nullptr;
            v.type = Json::NUM;
            v.num = std::strtod(digits.c_str(), &stop);
            if (stop != digits.c_str() + digits.size()) return fail("bad JSON number");
            if (!std::isfinite(v.num)) return fail("JSON number out of range");
        }
        --depth;
        return ok;
    }
};

int json_vec3(const Json& root, const char* key, float out[3], const std::string& path) {
    const Json* v = root.get(key);
    if (!v || v->type != Json::ARR || v->arr.size() < 3)
        return set_error(CRT_ERR_INVALID, path + ": `" + key + "` must be an array of 3 numbers");
    for (int k = 0; k < 3; ++k) {
        if (v->arr[k].type != Json::NUM)
            return set_error(CRT_ERR_INVALID, path + ": `" + key + "` must be an array of 3 numbers");
        out[k] = (float)v->arr[k].num;
    }
    return CRT_OK;
}

int json_number(const Json& root, const char* key, float& out, const std::string& path) {
    const Json* v = root.get(key);
    if (!v || v->type != Json::NUM) return set_error(CRT_ERR_INVALID, path + ": `" + key + "` must be a number");
    out = (float)v->num;
    return CRT_OK;
}

// ---------------------------------------------------------------------------
// scene assembly
// ---------------------------------------------------------------------------
int load_scene_files(const std::string& obj_path, const std::string& texture_dir, uint32_t flags,
                     crt_scene_files_s& S) {
    const auto t0 = Clock::now();
    if (!ends_with(obj_path, ".obj")) return set_error(CRT_ERR_INVALID, "scene file is not a .obj file: " + obj_path);
    FileView text;
    std::string err;
    if (!map_file(obj_path, text, err)) return set_error(CRT_ERR_INVALID, err);
    S.info.file_bytes = text.size;
    const char* base = text.data;
    const char* end = base + text.size;

    // line-aligned chunks of ~4 MB (at least one per thread for large files)
    const size_t hw = std::max(1u, std::thread::hardware_concurrency());
    const size_t want = std::max<size_t>(1, std::min(text.size / (1u << 16) + 1,
                                                     std::max(hw * 4, text.size / (4u << 20) + 1)));
    std::vector<Chunk> chunks;
    {
        const char* p = base;
        for (size_t k = 0; k < want && p < end; ++k) {
            const char* q = k + 1 == want ? end : base + (text.size * (k + 1)) / want;
            if (q < p) q = p;
            if (q < end) {
                const char* nl = static_cast<const char*>(std::memchr(q, '\n', (size_t)(end - q)));
                q = nl ? nl + 1 : end;
            }
            Chunk c;
            c.b = p;
            c.e = q;
            chunks.push_back(std::move(c));
            p = q;
        }
        if (chunks.empty()) {
            Chunk c;
            c.b = c.e = base;
            chunks.push_back(std::move(c));
        }
    }

    // pass 1: classify lines, count records and triangles, note events
    parallel_for(chunks.size(), [&](size_t ci) {
        Chunk& C = chunks[ci];
        for (const char* p = C.b; p < C.e;) {
            LineText L;
            p = next_line(p, C.e, L);
            ++C.lines;
            switch (classify(L)) {
                case L_V: ++C.nv; break;
                case L_VT: ++C.nvt; break;
                case L_VN: ++C.nvn; break;
                case L_F: {
                    const int k = count_face_vertices(L.tail);
                    if (k < 3) {
                        C.fail(C.lines, "face with fewer than 3 vertices");
                        return;
                    }
                    C.ntri += (uint64_t)(k - 2);
                    if (k > 3) ++C.npoly;
                    break;
                }
                case L_GROUP:
                    C.events.push_back({L_GROUP, L.head == "o" || L.head == "g", C.ntri, std::string(L.tail)});
                    break;
                case L_USEMTL:
                    C.events.push_back({L_USEMTL, false, C.ntri, std::string(L.tail)});
                    break;
                case L_MTLLIB:
                    C.events.push_back({L_MTLLIB, false, C.ntri, std::string(L.tail)});
                    break;
                default: break;
            }
        }
    });
    uint64_t nv = 0, nvt = 0, nvn = 0, ntri = 0, lines = 0, npoly = 0;
    for (Chunk& C : chunks) {
        C.line0 = lines; C.v0 = nv; C.vt0 = nvt; C.vn0 = nvn; C.tri0 = ntri;
        lines += C.lines; nv += C.nv; nvt += C.nvt; nvn += C.nvn; ntri += C.ntri; npoly += C.npoly;
    }
    auto first_error = [&]() -> int {
        for (Chunk& C : chunks)
            if (!C.err.empty())
                return set_error(CRT_ERR_INVALID, obj_path + ":" + std::to_string(C.err_line) + ": " + C.err);
        return CRT_OK;
    };
    // line numbers of pass-1 errors are chunk-local until line0 is known
    for (Chunk& C : chunks)
        if (!C.err.empty()) C.err_line += C.line0;
    if (int st = first_error()) return st;
    if (ntri == 0) return set_error(CRT_ERR_INVALID, obj_path + ": no faces");
    if (ntri >= (1ull << 31)) return set_error(CRT_ERR_LIMIT, obj_path + ": more than 2^31 triangles");

    // pass 2: v / vt / vn records
    RawArray<float> P, T, N;
    P.allocate(3 * nv);
    T.allocate(2 * nvt);
    N.allocate(3 * nvn);
    parallel_for(chunks.size(), [&](size_t ci) {
        Chunk& C = chunks[ci];
        uint64_t iv = C.v0, ivt = C.vt0, ivn = C.vn0, line = 0;
        for (const char* p = C.b; p < C.e;) {
            LineText L;
            p = next_line(p, C.e, L);
            ++line;
            const LineKind k = classify(L);
            if (k != L_V && k != L_VT && k != L_VN) continue;
            const char* q = L.tail.data();
            const char* qe = q + L.tail.size();
            const int want_n = k == L_VT ? 2 : 3;
            float v[3] = {0, 0, 0};
            int got = 0;
            for (std::string_view tok; got < want_n && !(tok = next_token(q, qe)).empty(); ++got) {
                if (!parse_float(tok, v[got])) {
                    C.fail(line, "bad number `" + std::string(tok) + "`");
                    return;
                }
            }
            // a texture coordinate may omit v (0); positions and normals need 3
            if (got < (k == L_VT ? 1 : 3)) {
                C.fail(line, "too few values");
                return;
            }
            if (k == L_V) std::memcpy(&P[3 * iv++], v, 3 * sizeof(float));
            else if (k == L_VT) std::memcpy(&T[2 * ivt++], v, 2 * sizeof(float));
            else std::memcpy(&N[3 * ivn++], v, 3 * sizeof(float));
        }
    });
    if (int st = first_error()) return st;

    // pass 3: faces, fanned into triangles (0, j, j + 1)
    S.positions.allocate(9 * ntri);
    S.normals.allocate(9 * ntri);
    S.uvs.allocate(6 * ntri);
    parallel_for(chunks.size(), [&](size_t ci) {
        Chunk& C = chunks[ci];
        uint64_t cv = C.v0, cvt = C.vt0, cvn = C.vn0, tri = C.tri0, line = 0;
        std::vector<FaceVertex> fv;
        std::vector<float> vp, vn, vt;
        for (const char* p = C.b; p < C.e;) {
            LineText L;
            p = next_line(p, C.e, L);
            ++line;
            switch (classify(L)) {
                case L_V: ++cv; continue;
                case L_VT: ++cvt; continue;
                case L_VN: ++cvn; continue;
                case L_F: break;
                default: continue;
            }
            fv.clear();
            bool all_normals = true;
            const char* q = L.tail.data();
            const char* qe = q + L.tail.size();
            for (std::string_view tok; !(tok = next_token(q, qe)).empty();) {
                FaceVertex x;
                if (!parse_face_vertex(tok, cv, cvt, cvn, x)) {
                    C.fail(line, "bad face vertex `" + std::string(tok) + "`");
                    return;
                }
                all_normals = all_normals && x.n >= 0;
                fv.push_back(x);
            }
            const size_t k = fv.size();
            vp.resize(3 * k);
            vn.resize(3 * k);
            vt.resize(2 * k);
            for (size_t j = 0; j < k; ++j) {
                std::memcpy(&vp[3 * j], &P[3 * fv[j].p], 3 * sizeof(float));
                if (fv[j].t >= 0) std::memcpy(&vt[2 * j], &T[2 * fv[j].t], 2 * sizeof(float));
                else vt[2 * j] = vt[2 * j + 1] = 0.f;
                if (fv[j].n >= 0) std::memcpy(&vn[3 * j], &N[3 * fv[j].n], 3 * sizeof(float));
            }
            if (!all_normals) {
                // a face with any vertex lacking a normal gets the unnormalised
                // (p0 - p1) x (p2 - p1) on every vertex (obj_load.h:832-843)
                const float A[3] = {vp[0] - vp[3], vp[1] - vp[4], vp[2] - vp[5]};
                const float B[3] = {vp[6] - vp[3], vp[7] - vp[4], vp[8] - vp[5]};
                const float c[3] = {A[1] * B[2] - A[2] * B[1], A[2] * B[0] - A[0] * B[2],
                                    A[0] * B[1] - A[1] * B[0]};
                for (size_t j = 0; j < k; ++j) std::memcpy(&vn[3 * j], c, sizeof c);
            }
            for (size_t j = 1; j + 1 < k; ++j, ++tri) {
                const size_t corner[3] = {0, j, j + 1};
                for (int c = 0; c < 3; ++c) {
                    std::memcpy(&S.positions[9 * tri + 3 * c], &vp[3 * corner[c]], 3 * sizeof(float));
                    std::memcpy(&S.normals[9 * tri + 3 * c], &vn[3 * corner[c]], 3 * sizeof(float));
                    std::memcpy(&S.uvs[6 * tri + 2 * c], &vt[2 * corner[c]], 2 * sizeof(float));
                }
            }
        }
    });
    if (int st = first_error()) return st;

    // meshes and material names in file order (LoadFile's grouping rules:
    // the first o/g only names the open mesh; later ones and every usemtl
    // close a non-empty mesh; mesh i takes the i-th usemtl name)
    std::vector<MtlMaterial> mtl;
    std::vector<std::string> mesh_mtl;
    std::string dir;
    {
        const size_t slash = obj_path.rfind('/');
        if (slash != std::string::npos) dir = obj_path.substr(0, slash + 1);
    }
    bool listening = false;
    uint64_t mesh_start = 0;
    std::string name;
    for (const Chunk& C : chunks) {
        for (const Event& ev : C.events) {
            const uint64_t at = C.tri0 + ev.tri;
            if (ev.kind == L_GROUP) {
                if (listening && at > mesh_start) {
                    S.meshes.push_back({name, (uint32_t)mesh_start, (uint32_t)(at - mesh_start)});
                    mesh_start = at;
                    name = ev.text;
                } else {
                    name = ev.named ? ev.text : std::string("unnamed");
                }
                listening = true;
            } else if (ev.kind == L_USEMTL) {
                mesh_mtl.push_back(ev.text);
                if (at > mesh_start) {
                    S.meshes.push_back({name + "_2", (uint32_t)mesh_start, (uint32_t)(at - mesh_start)});
                    mesh_start = at;
                }
            } else {
                if (int st = load_mtl(dir + ev.text, mtl, S.info.file_bytes)) return st;
            }
        }
    }
    if (ntri > mesh_start) S.meshes.push_back({name, (uint32_t)mesh_start, (uint32_t)(ntri - mesh_start)});
    S.info.parse_ms = (float)ms_since(t0);

    // textures: every distinct map_Kd of the libraries, in library order
    // (Scene::loadTextures, scene.cpp:55-71)
    const auto t1 = Clock::now();
    std::vector<std::string> tex_files;
    for (const MtlMaterial& m : mtl)
        if (!m.map_Kd.empty() && std::find(tex_files.begin(), tex_files.end(), m.map_Kd) == tex_files.end())
            tex_files.push_back(m.map_Kd);
    std::string tdir = texture_dir;
    if (!tdir.empty() && tdir.back() != '/') tdir.push_back('/');
    std::vector<Png> images(tex_files.size());
    std::vector<std::string> tex_err(tex_files.size());
    std::vector<uint64_t> tex_bytes(tex_files.size(), 0);
    parallel_for(tex_files.size(), [&](size_t k) {
        std::string bytes, e;
        const std::string path = tdir + tex_files[k];
        if (!read_file(path, bytes, e)) {
            tex_err[k] = e;
            return;
        }
        tex_bytes[k] = bytes.size();
        if (!decode_png(bytes, images[k], e)) tex_err[k] = path + ": " + e;
    });
    for (size_t k = 0; k < tex_files.size(); ++k) {
        if (!tex_err[k].empty()) return set_error(CRT_ERR_INVALID, tex_err[k]);
        S.info.file_bytes += tex_bytes[k];
    }
    uint64_t total_texels = 0;
    for (const Png& im : images) total_texels += (uint64_t)im.w * im.h;
    if (total_texels >= (1ull << 32)) return set_error(CRT_ERR_LIMIT, "textures hold 2^32 texels or more");
    S.texels.resize(3 * total_texels);
    {
        const float* lut = gamma_lut();
        uint64_t off = 0;
        for (const Png& im : images) {
            S.texture_dims.push_back(im.w);
            S.texture_dims.push_back(im.h);
            const size_t cnt = (size_t)im.w * im.h * 3;
            float* dst = S.texels.data() + 3 * off;
            for (size_t i = 0; i < cnt; ++i) dst[i] = lut[im.rgb[i]];
            off += (uint64_t)im.w * im.h;
        }
    }
    S.info.texture_ms = (float)ms_since(t1);

    // material table and per-face ids (Scene::loadTriangles, scene.cpp:74-104)
    const MtlMaterial fallback;   // objl::Mesh's default MeshMaterial
    std::vector<int64_t> mesh_src(S.meshes.size(), -1);   // index into mtl, -1 = fallback
    for (size_t i = 0; i < S.meshes.size() && i < mesh_mtl.size(); ++i)
        for (size_t j = 0; j < mtl.size(); ++j)
            if (mtl[j].name == mesh_mtl[i]) {
                mesh_src[i] = (int64_t)j;
                break;
            }
    auto src_of = [&](size_t i) -> const MtlMaterial& { return mesh_src[i] < 0 ? fallback : mtl[mesh_src[i]]; };
    auto texture_of = [&](const MtlMaterial& m) -> int32_t {
        if (m.map_Kd.empty()) return CRT_NO_TEXTURE;
        return (int32_t)(std::find(tex_files.begin(), tex_files.end(), m.map_Kd) - tex_files.begin());
    };
    std::vector<uint32_t> mesh_id(S.meshes.size());
    std::vector<TableMaterial> table;
    if (flags & CRT_LOAD_EXACT_MATERIALS) {
        std::vector<int64_t> seen;
        for (size_t i = 0; i < S.meshes.size(); ++i) {
            auto it = std::find(seen.begin(), seen.end(), mesh_src[i]);
            if (it == seen.end()) {
                seen.push_back(mesh_src[i]);
                TableMaterial t = table_material(src_of(i));
                t.texture = texture_of(src_of(i));
                table.push_back(t);
                it = seen.end() - 1;
            }
            mesh_id[i] = (uint32_t)(it - seen.begin());
        }
    } else {
        // populateMaterialsMap (scene.cpp:192-203): the index counts every
        // material the map did not find, whether or not the insert took it.
        // With an inconsistent order the tree's shape decides what merges,
        // so the inserts must take libstdc++'s plain unique-insert descent,
        // as the reference's C++14 insert(pair) does: insert(const
        // value_type&).  (C++17's emplace and insert(P&&) first look up
        // lower_bound and insert at that hint, which with this order can
        // drop nodes from the tree.)
        using Merged = std::map<TableMaterial, uint32_t, ReferenceOrder>;
        Merged merged;
        uint32_t next = 0;
        for (size_t i = 0; i < S.meshes.size(); ++i) {
            const TableMaterial t = table_material(src_of(i));
            if (merged.count(t) == 0) {
                const Merged::value_type entry(t, next++);
                merged.insert(entry);
            }
        }
        if (next != merged.size())
            return set_error(CRT_ERR_INVALID, obj_path + ": materials collide in the reference's "
                             "material merge (its table would be written out of bounds)");
        table.resize(merged.size());
        for (const auto& kv : merged) table[kv.second] = kv.first;
        for (size_t i = 0; i < S.meshes.size(); ++i) {
            const TableMaterial t = table_material(src_of(i));
            size_t id = 0;
            while (id < table.size() && !reference_equal(table[id], t)) ++id;
            // the reference indexes one past its table when nothing compares
            // equal (a material that differs only in `diffuse` from a merged
            // one); the merged entry is taken instead
            if (id == table.size()) {
                auto it = merged.find(t);
                if (it == merged.end())
                    return set_error(CRT_ERR_INVALID, obj_path + ": a mesh's material has no entry "
                                     "in the reference's material merge");
                id = it->second;
            }
            mesh_id[i] = (uint32_t)id;
            const int32_t tex = texture_of(src_of(i));
            if (tex != CRT_NO_TEXTURE) table[id].texture = tex;   // the last mesh wins
        }
    }
    for (const TableMaterial& t : table) S.materials.push_back(to_abi(t));
    S.material_ids.assign(ntri, 0);
    parallel_for(S.meshes.size(), [&](size_t i) {
        std::fill(S.material_ids.begin() + S.meshes[i].first,
                  S.material_ids.begin() + S.meshes[i].first + S.meshes[i].count, mesh_id[i]);
    });

    crt_scene_files_info& I = S.info;
    I.num_triangles = (uint32_t)ntri;
    I.num_meshes = (uint32_t)S.meshes.size();
    I.num_materials = (uint32_t)S.materials.size();
    I.num_mtl_materials = (uint32_t)mtl.size();
    I.num_textures = (uint32_t)images.size();
    I.num_positions = (uint32_t)nv;
    I.num_texcoords = (uint32_t)nvt;
    I.num_normals = (uint32_t)nvn;
    I.num_polygons = (uint32_t)npoly;
    return CRT_OK;
}

}  // namespace

extern "C" {

int crt_scene_files_load(const char* obj_path, const char* texture_dir, uint32_t flags, crt_scene_files* out) {
    if (!obj_path || !out) return set_error(CRT_ERR_INVALID, "crt_scene_files_load: null argument");
    *out = nullptr;
    if (flags & ~(uint32_t)CRT_LOAD_EXACT_MATERIALS) return set_error(CRT_ERR_INVALID, "crt_scene_files_load: unknown flags");
    try {
        std::unique_ptr<crt_scene_files_s> S(new crt_scene_files_s);
        if (int st = load_scene_files(obj_path, texture_dir ? texture_dir : "", flags, *S)) return st;
        *out = S.release();
        return CRT_OK;
    } catch (const std::bad_alloc&) {
        return set_error(CRT_ERR_NOMEM, "crt_scene_files_load: out of host memory");
    } catch (const std::exception& e) {
        return set_error(CRT_ERR_INVALID, std::string("crt_scene_files_load: ") + e.what());
    }
}

int crt_scene_files_desc(crt_scene_files f, crt_scene_desc* d) {
    if (!f || !d) return set_error(CRT_ERR_INVALID, "crt_scene_files_desc: null argument");
    std::memset(d, 0, sizeof *d);
    d->num_triangles = f->info.num_triangles;
    d->positions = f->positions.data();
    d->normals = f->normals.data();
    d->uvs = f->uvs.data();
    d->material_ids = f->material_ids.data();
    d->num_materials = (uint32_t)f->materials.size();
    d->materials = f->materials.data();
    d->num_textures = f->info.num_textures;
    d->texture_dims = f->texture_dims.empty() ? nullptr : f->texture_dims.data();
    d->texels = f->texels.empty() ? nullptr : f->texels.data();
    return CRT_OK;
}

int crt_scene_files_get_info(crt_scene_files f, crt_scene_files_info* out) {
    if (!f || !out) return set_error(CRT_ERR_INVALID, "crt_scene_files_get_info: null argument");
    *out = f->info;
    return CRT_OK;
}

int crt_scene_files_mesh(crt_scene_files f, uint32_t mesh, const char** name, uint32_t* first_triangle,
                         uint32_t* num_triangles) {
    if (!f) return set_error(CRT_ERR_INVALID, "crt_scene_files_mesh: null argument");
    if (mesh >= f->meshes.size()) return set_error(CRT_ERR_INVALID, "crt_scene_files_mesh: no such mesh");
    if (name) *name = f->meshes[mesh].name.c_str();
    if (first_triangle) *first_triangle = f->meshes[mesh].first;
    if (num_triangles) *num_triangles = f->meshes[mesh].count;
    return CRT_OK;
}

int crt_scene_files_destroy(crt_scene_files f) {
    delete f;
    return CRT_OK;
}

int crt_camera_load_json(const char* path, uint32_t width, uint32_t height, crt_camera* out) {
    if (!path || !out) return set_error(CRT_ERR_INVALID, "crt_camera_load_json: null argument");
    try {
        std::string text, err;
        if (!read_file(path, text, err)) return set_error(CRT_ERR_INVALID, err);
        JsonParser jp(text.data(), text.data() + text.size());
        Json root;
        if (!jp.value(root)) return set_error(CRT_ERR_INVALID, std::string(path) + ": " + jp.err);
        jp.ws();
        if (jp.p != jp.e) return set_error(CRT_ERR_INVALID, std::string(path) + ": trailing characters after JSON");
        if (root.type != Json::OBJ) return set_error(CRT_ERR_INVALID, std::string(path) + ": not a JSON object");
        float fov, focal, fstop, eye[3], dir[3], up[3];
        const std::string p(path);
        if (int st = json_number(root, "fieldOfView", fov, p)) return st;
        if (int st = json_number(root, "focalLength", focal, p)) return st;
        if (int st = json_number(root, "fStop", fstop, p)) return st;
        if (int st = json_vec3(root, "eye", eye, p)) return st;
        if (int st = json_vec3(root, "viewDirection", dir, p)) return st;
        if (int st = json_vec3(root, "upDirection", up, p)) return st;
        return crt_camera_from_json(fov, focal, fstop, eye, dir, up, width, height, out);
    } catch (const std::exception& e) {
        return set_error(CRT_ERR_INVALID, std::string("crt_camera_load_json: ") + e.what());
    }
}

int crt_texture_load_png(const char* path, uint32_t dims[2], float* texels, uint64_t capacity) {
    if (!path || !dims) return set_error(CRT_ERR_INVALID, "crt_texture_load_png: null argument");
    try {
        std::string bytes, err;
        if (!read_file(path, bytes, err)) return set_error(CRT_ERR_INVALID, err);
        Png im;
        if (!decode_png(bytes, im, err)) return set_error(CRT_ERR_INVALID, std::string(path) + ": " + err);
        dims[0] = im.w;
        dims[1] = im.h;
        if (!texels) return CRT_OK;
        if (capacity < (uint64_t)im.w * im.h)
            return set_error(CRT_ERR_INVALID, "crt_texture_load_png: texel buffer too small");
        const float* lut = gamma_lut();
        for (size_t i = 0; i < im.rgb.size(); ++i) texels[i] = lut[im.rgb[i]];
        return CRT_OK;
    } catch (const std::bad_alloc&) {
        return set_error(CRT_ERR_NOMEM, "crt_texture_load_png: out of host memory");
    }
}

int crt_image_write_png(const char* path, uint32_t width, uint32_t height, const uint8_t* rgba) {
    if (!path || !rgba || width == 0 || height == 0)
        return set_error(CRT_ERR_INVALID, "crt_image_write_png: bad argument");
    if (((uint64_t)width * 4 + 1) * height >= (1ull << 31))
        return set_error(CRT_ERR_LIMIT, "crt_image_write_png: image too large");
    try {
        const std::vector<uint8_t> png = encode_png(width, height, rgba);
        FILE* f = std::fopen(path, "wb");
        if (!f) return set_error(CRT_ERR_INVALID, std::string("cannot write ") + path);
        const size_t put = std::fwrite(png.data(), 1, png.size(), f);
        const int closed = std::fclose(f);
        if (put != png.size() || closed != 0) return set_error(CRT_ERR_INVALID, std::string("short write of ") + path);
        return CRT_OK;
    } catch (const std::bad_alloc&) {
        return set_error(CRT_ERR_NOMEM, "crt_image_write_png: out of host memory");
    }
}

}  // extern "C"
