// Circuit file loaders of the reference (host only): the binary CIRCUIT2 segment format
// read by CircuitRaw (include/circuit/circuit_raw.hpp:437-607) and flattened by
// Circuit::from_circuit_raw (include/circuit/circuit.hpp:217-251), and the text gate lists
// of Circuit::load_extracted_gates (circuit.hpp:152-215).
//
// Behaviour kept from the reference, because proofs of a loaded circuit must match:
//  - a CIRCUIT2 field element is 32 bytes on disk and the reference's M31 reader sets it
//    to 1 whatever the bytes are (M31::operator>>, include/field/M31.hpp:124-135), so every
//    gate coefficient of a CIRCUIT2 circuit is 1 (random-coefficient gates included: their
//    sentinel is replaced by the file's rand_sentinel, which reads as 1 too);
//  - const gates are dropped (from_circuit_raw flattens only mul and add gates);
//  - a layer's sizes come from its largest gate ids, not from the segment lengths:
//    nb_vars = ctz(next_pow_of_2(max_id)), with next_pow_of_2(2^k) = 2^k and 0 for
//    max_id = 0 (_compute_nb_vars, circuit.hpp:124-150, include/utils/myutil.hpp:38-48).
//    A file whose largest id is an exact power of two therefore gets a layer one bit too
//    narrow, as in the reference; circuit upload rejects it (id out of range) instead of
//    reading past the table as the reference would.
// Gate order inside a layer follows the segment tree walk; it does not affect proofs
// (every round value is a field sum).
#include <stdint.h>
#include <string.h>

#include <algorithm>
#include <cstdlib>
#include <map>
#include <new>
#include <string>
#include <utility>
#include <vector>

#include "../../include/gkrgpu.h"

namespace gkrgpu {
void set_last_error(const char* msg);
}

struct gkrgpu_parsed {
    struct Layer {
        uint32_t nb_in = 0, nb_out = 0;
        std::vector<gkrgpu_mul_gate> mul;
        std::vector<gkrgpu_add_gate> add;
    };
    std::vector<Layer> layers;
};

namespace {

constexpr uint64_t kMagic = 3626604230490605891ull;  // "CIRCUIT2" read as a little-endian u64

struct ParseError {
    std::string msg;
};

class Reader {
   public:
    Reader(const uint8_t* p, uint64_t n) : p_(p), n_(n) {}
    uint64_t u64() {
        need(8);
        uint64_t x = 0;
        for (int k = 7; k >= 0; k--) x = (x << 8) | p_[off_ + k];
        off_ += 8;
        return x;
    }
    void field() { need(32), off_ += 32; }  // 32-byte element; the reference keeps 1
    // a count that must fit in what is left of the file at `unit` bytes per item
    uint64_t count(uint64_t unit, const char* what) {
        const uint64_t c = u64();
        if (unit && c > (n_ - off_) / unit) throw ParseError{std::string("truncated file: ") + what + " count too large"};
        return c;
    }
    uint64_t offset() const { return off_; }

   private:
    void need(uint64_t k) {
        if (n_ - off_ < k) throw ParseError{"truncated file"};
    }
    const uint8_t* p_;
    uint64_t n_, off_ = 0;
};

struct Seg {
    uint64_t i_len = 0, o_len = 0;
    std::vector<std::pair<uint64_t, std::vector<std::pair<uint64_t, uint64_t>>>> children;  // (id, (i_off, o_off))
    std::vector<uint64_t> mul;  // in0, in1, out
    std::vector<uint64_t> add;  // in0, out
    bool has_gates = false;     // mul, add or const gates present (a leaf of the walk)
};

// Segment (circuit_raw.hpp:275-352).
Seg read_segment(Reader& r) {
    Seg s;
    s.i_len = r.u64();
    s.o_len = r.u64();
    const uint64_t nc = r.count(16, "child segment");
    s.children.resize(nc);
    for (uint64_t i = 0; i < nc; i++) {
        s.children[i].first = r.u64();
        const uint64_t na = r.count(16, "allocation");
        s.children[i].second.resize(na);
        for (uint64_t j = 0; j < na; j++) {
            s.children[i].second[j].first = r.u64();
            s.children[i].second[j].second = r.u64();
        }
    }
    const uint64_t nm = r.count(56, "mul gate");
    s.mul.reserve(3 * nm);
    for (uint64_t i = 0; i < nm; i++) {
        s.mul.push_back(r.u64());
        s.mul.push_back(r.u64());
        s.mul.push_back(r.u64());
        r.field();
    }
    const uint64_t na = r.count(48, "add gate");
    s.add.reserve(2 * na);
    for (uint64_t i = 0; i < na; i++) {
        s.add.push_back(r.u64());
        s.add.push_back(r.u64());
        r.field();
    }
    const uint64_t nk = r.count(40, "const gate");
    for (uint64_t i = 0; i < nk; i++) {
        r.u64();
        r.field();
    }
    const uint64_t nr = r.count(8, "random coefficient index");
    for (uint64_t i = 0; i < nr; i++)
        if (r.u64() >= nm + na + nk) throw ParseError{"random coefficient index out of range"};
    s.has_gates = nm || na || nk;
    return s;
}

// scan_leaf_segments (circuit_raw.hpp:81-117): every gate-holding segment under `cur` with
// the (input, output) offsets of each of its placements.
using Leaves = std::map<uint64_t, std::vector<std::pair<uint64_t, uint64_t>>>;

Leaves scan_leaves(const std::vector<Seg>& segs, uint64_t cur, int depth) {
    if (depth > 256) throw ParseError{"segment nesting deeper than 256 (cyclic segment references?)"};
    Leaves ret;
    const Seg& s = segs[cur];
    if (s.has_gates) ret[cur].push_back({0, 0});
    for (const auto& child : s.children) {
        if (child.first >= segs.size()) throw ParseError{"child segment id out of range"};
        const Leaves sub = scan_leaves(segs, child.first, depth + 1);
        for (const auto& leaf : sub)
            for (const auto& la : leaf.second)
                for (const auto& ca : child.second) ret[leaf.first].push_back({ca.first + la.first, ca.second + la.second});
    }
    return ret;
}

uint32_t next_pow_of_2(uint32_t n) {
    if (n == 0 || (n & (n - 1)) == 0) return n;
    uint32_t p = 1;
    while (p < n) p <<= 1;
    return p;
}

// _compute_nb_vars (circuit.hpp:124-150) for one layer.
void compute_nb_vars(gkrgpu_parsed::Layer& L) {
    uint32_t mo = 0, mi = 0;
    for (const auto& g : L.mul) {
        mo = std::max(mo, g.o_id);
        mi = std::max({mi, g.i0, g.i1});
    }
    for (const auto& g : L.add) {
        mo = std::max(mo, g.o_id);
        mi = std::max(mi, g.i0);
    }
    L.nb_in = mi ? (uint32_t)__builtin_ctz(next_pow_of_2(mi)) : 0u;
    L.nb_out = mo ? (uint32_t)__builtin_ctz(next_pow_of_2(mo)) : 0u;
}

uint32_t id32(uint64_t x) {
    if (x > 0xffffffffull) throw ParseError{"gate id does not fit in 32 bits"};
    return (uint32_t)x;
}

void parse_circuit2(const uint8_t* p, uint64_t n, gkrgpu_parsed& out) {
    Reader r(p, n);
    if (r.u64() != kMagic) throw ParseError{"not a CIRCUIT2 file (bad magic number)"};
    const uint64_t ns = r.count(48, "segment");
    std::vector<Seg> segs(ns);
    for (uint64_t i = 0; i < ns; i++) segs[i] = read_segment(r);
    const uint64_t nl = r.count(8, "layer");
    std::vector<uint64_t> layer_seg(nl);
    for (uint64_t i = 0; i < nl; i++) {
        layer_seg[i] = r.u64();
        if (layer_seg[i] >= ns) throw ParseError{"layer segment id out of range"};
    }
    r.field();  // rand_sentinel
    out.layers.assign(nl, {});
    for (uint64_t l = 0; l < nl; l++) {
        const Leaves leaves = scan_leaves(segs, layer_seg[l], 0);
        auto& L = out.layers[l];
        for (const auto& leaf : leaves) {
            const Seg& s = segs[leaf.first];
            for (const auto& a : leaf.second) {
                for (size_t k = 0; k < s.mul.size(); k += 3)
                    L.mul.push_back({id32(s.mul[k + 2] + a.second), id32(s.mul[k] + a.first), id32(s.mul[k + 1] + a.first), 1u});
                for (size_t k = 0; k < s.add.size(); k += 2)
                    L.add.push_back({id32(s.add[k + 1] + a.second), id32(s.add[k] + a.first), 1u});
            }
        }
        compute_nb_vars(L);
    }
}

// load_extracted_gates (circuit.hpp:152-215): line i of each file holds the gate count then
// the gates of layer (lines - 1 - i): mul "in0 in1 out coef", add "in0 out coef".  Coefficients
// are reduced mod 2^31 - 1 (M31's constructor from an integer).
class Text {
   public:
    Text(const char* p, uint64_t n) : p_(p), n_(n) {}
    bool eof() {
        skip();
        return off_ >= n_;
    }
    uint64_t num() {
        skip();
        if (off_ >= n_ || p_[off_] < '0' || p_[off_] > '9') throw ParseError{"expected a number"};
        uint64_t x = 0;
        while (off_ < n_ && p_[off_] >= '0' && p_[off_] <= '9') {
            const uint64_t d = (uint64_t)(p_[off_++] - '0');
            if (x > (~0ull - d) / 10) throw ParseError{"number too large"};
            x = 10 * x + d;
        }
        return x;
    }
    // lines as std::getline counts them (a last line without '\n' counts)
    uint64_t lines() const {
        uint64_t c = 0;
        for (uint64_t i = 0; i < n_; i++) c += p_[i] == '\n';
        return c + (n_ && p_[n_ - 1] != '\n');
    }

   private:
    void skip() {
        while (off_ < n_ && (p_[off_] == ' ' || p_[off_] == '\n' || p_[off_] == '\r' || p_[off_] == '\t')) off_++;
    }
    const char* p_;
    uint64_t n_, off_ = 0;
};

uint32_t m31_coef(uint64_t c) {
    if (c > 0xffffffffull) throw ParseError{"coefficient does not fit in 32 bits"};
    uint32_t x = (uint32_t)c;
    x = (x & 0x7fffffffu) + (x >> 31);
    return x == 0x7fffffffu ? 0u : x;
}

void parse_extracted(const char* mul, uint64_t nm, const char* add, uint64_t na, gkrgpu_parsed& out) {
    Text tm(mul, nm), ta(add, na);
    const uint64_t nl = tm.lines();
    if (nl == 0 || nl > 4096) throw ParseError{"the mul file must hold 1..4096 lines"};
    out.layers.assign(nl, {});
    for (uint64_t i = 0; i < nl; i++) {
        auto& L = out.layers[nl - 1 - i];
        const uint64_t g = tm.num();
        if (g > nm) throw ParseError{"mul gate count larger than the file"};
        for (uint64_t k = 0; k < g; k++) {
            const uint32_t i0 = id32(tm.num()), i1 = id32(tm.num()), o = id32(tm.num());
            L.mul.push_back({o, i0, i1, m31_coef(tm.num())});
        }
    }
    for (uint64_t i = 0; i < nl; i++) {
        auto& L = out.layers[nl - 1 - i];
        if (ta.eof()) throw ParseError{"the add file has fewer layers than the mul file"};
        const uint64_t g = ta.num();
        if (g > na) throw ParseError{"add gate count larger than the file"};
        for (uint64_t k = 0; k < g; k++) {
            const uint32_t i0 = id32(ta.num()), o = id32(ta.num());
            L.add.push_back({o, i0, m31_coef(ta.num())});
        }
    }
    for (auto& L : out.layers) compute_nb_vars(L);
}

template <class F>
int parse_guarded(gkrgpu_parsed** out, F&& f) {
    if (!out) {
        gkrgpu::set_last_error("null output");
        return GKRGPU_ERR_INVALID;
    }
    *out = nullptr;
    gkrgpu_parsed* c = new (std::nothrow) gkrgpu_parsed();
    if (!c) {
        gkrgpu::set_last_error("host allocation failed");
        return GKRGPU_ERR_NOMEM;
    }
    try {
        f(*c);
    } catch (const ParseError& e) {
        delete c;
        gkrgpu::set_last_error(e.msg.c_str());
        return GKRGPU_ERR_INVALID;
    } catch (const std::bad_alloc&) {
        delete c;
        gkrgpu::set_last_error("host allocation failed");
        return GKRGPU_ERR_NOMEM;
    }
    *out = c;
    return GKRGPU_OK;
}

}  // namespace

extern "C" {

int gkrgpu_circuit2_parse(const uint8_t* bytes, uint64_t len, gkrgpu_parsed** out) {
    if (!bytes && len) {
        gkrgpu::set_last_error("null buffer");
        return GKRGPU_ERR_INVALID;
    }
    return parse_guarded(out, [&](gkrgpu_parsed& c) { parse_circuit2(bytes, len, c); });
}

int gkrgpu_extracted_parse(const char* mul_text, uint64_t mul_len, const char* add_text, uint64_t add_len,
                           gkrgpu_parsed** out) {
    if ((!mul_text && mul_len) || (!add_text && add_len)) {
        gkrgpu::set_last_error("null buffer");
        return GKRGPU_ERR_INVALID;
    }
    return parse_guarded(out, [&](gkrgpu_parsed& c) { parse_extracted(mul_text, mul_len, add_text, add_len, c); });
}

int gkrgpu_parsed_layers(const gkrgpu_parsed* parsed) { return parsed ? (int)parsed->layers.size() : -GKRGPU_ERR_INVALID; }

int gkrgpu_parsed_layer(const gkrgpu_parsed* parsed, int layer, gkrgpu_layer_desc* out) {
    if (!parsed || !out || layer < 0 || layer >= (int)parsed->layers.size()) {
        gkrgpu::set_last_error("null handle or layer index out of range");
        return GKRGPU_ERR_INVALID;
    }
    const auto& L = parsed->layers[layer];
    out->nb_input_vars = L.nb_in;
    out->nb_output_vars = L.nb_out;
    out->n_mul = L.mul.size();
    out->n_add = L.add.size();
    out->mul = L.mul.empty() ? nullptr : L.mul.data();
    out->add = L.add.empty() ? nullptr : L.add.data();
    return GKRGPU_OK;
}

void gkrgpu_parsed_free(gkrgpu_parsed* parsed) { delete parsed; }

}  // extern "C"
