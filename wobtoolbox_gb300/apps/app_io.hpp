// Inputs of the JSON apps, written for this engine: a small JSON reader (the subset the configs
// use: objects, arrays, strings, numbers, booleans, null), a Wavefront OBJ reader (v / f lines,
// 1-based or negative indices, "i/t/n" corners, polygons fanned into triangles) and generalised
// winding numbers of segment and triangle soups -- the roles nlohmann::json, igl::readOBJ and
// igl::winding_number play for apps/general_2d.cu / general_3d.cu.
#pragma once

#include <cmath>
#include <cstdint>
#include <cstdlib>
#include <fstream>
#include <map>
#include <memory>
#include <sstream>
#include <stdexcept>
#include <string>
#include <vector>

namespace wobapp {

// ------------------------------------------------------------------ JSON
struct Json {
    enum Kind { Null, Bool, Number, String, Array, Object } kind = Null;
    bool b = false;
    double num = 0.0;
    std::string str;
    std::vector<Json> arr;
    std::map<std::string, Json> obj;

    bool contains(const std::string &k) const { return kind == Object && obj.count(k) != 0; }
    const Json &operator[](const std::string &k) const {
        auto it = obj.find(k);
        if (kind != Object || it == obj.end()) throw std::runtime_error("config: missing key \"" + k + "\"");
        return it->second;
    }
    double number() const {
        if (kind != Number) throw std::runtime_error("config: expected a number");
        return num;
    }
    const std::string &string() const {
        if (kind != String) throw std::runtime_error("config: expected a string");
        return str;
    }
    bool boolean() const {
        if (kind != Bool) throw std::runtime_error("config: expected true or false");
        return b;
    }
};

class JsonParser {
  public:
    explicit JsonParser(const std::string &text) : s_(text) {}
    Json parse() {
        Json v = value();
        ws();
        if (i_ != s_.size()) fail("trailing characters");
        return v;
    }

  private:
    const std::string &s_;
    size_t i_ = 0;

    [[noreturn]] void fail(const char *what) const {
        throw std::runtime_error(std::string("JSON: ") + what + " at offset " + std::to_string(i_));
    }
    void ws() {
        while (i_ < s_.size() && (s_[i_] == ' ' || s_[i_] == '\t' || s_[i_] == '\n' || s_[i_] == '\r')) i_++;
    }
    bool lit(const char *w) {
        size_t n = 0;
        while (w[n]) n++;
        if (s_.compare(i_, n, w) == 0) {
            i_ += n;
            return true;
        }
        return false;
    }
    Json value() {
        ws();
        if (i_ >= s_.size()) fail("unexpected end");
        Json v;
        const char c = s_[i_];
        if (c == '{') {
            v.kind = Json::Object;
            i_++;
            ws();
            if (i_ < s_.size() && s_[i_] == '}') {
                i_++;
                return v;
            }
            for (;;) {
                ws();
                if (i_ >= s_.size() || s_[i_] != '"') fail("expected a key");
                std::string k = string_lit();
                ws();
                if (i_ >= s_.size() || s_[i_] != ':') fail("expected ':'");
                i_++;
                v.obj[k] = value();
                ws();
                if (i_ < s_.size() && s_[i_] == ',') { i_++; continue; }
                if (i_ < s_.size() && s_[i_] == '}') { i_++; return v; }
                fail("expected ',' or '}'");
            }
        }
        if (c == '[') {
            v.kind = Json::Array;
            i_++;
            ws();
            if (i_ < s_.size() && s_[i_] == ']') {
                i_++;
                return v;
            }
            for (;;) {
                v.arr.push_back(value());
                ws();
                if (i_ < s_.size() && s_[i_] == ',') { i_++; continue; }
                if (i_ < s_.size() && s_[i_] == ']') { i_++; return v; }
                fail("expected ',' or ']'");
            }
        }
        if (c == '"') {
            v.kind = Json::String;
            v.str = string_lit();
            return v;
        }
        if (lit("true")) { v.kind = Json::Bool; v.b = true; return v; }
        if (lit("false")) { v.kind = Json::Bool; v.b = false; return v; }
        if (lit("null")) return v;
        const char *start = s_.c_str() + i_;
        char *end = nullptr;
        v.num = std::strtod(start, &end);
        if (end == start) fail("unexpected character");
        i_ += (size_t)(end - start);
        v.kind = Json::Number;
        return v;
    }
    std::string string_lit() {
        i_++;  // opening quote
        std::string out;
        while (i_ < s_.size() && s_[i_] != '"') {
            char c = s_[i_++];
            if (c == '\\') {
                if (i_ >= s_.size()) fail("bad escape");
                const char e = s_[i_++];
                switch (e) {
                case 'n': out += '\n'; break;
                case 't': out += '\t'; break;
                case 'r': out += '\r'; break;
                case 'b': out += '\b'; break;
                case 'f': out += '\f'; break;
                case 'u': {
                    if (i_ + 4 > s_.size()) fail("bad \\u escape");
                    const unsigned cp = (unsigned)std::strtoul(s_.substr(i_, 4).c_str(), nullptr, 16);
                    i_ += 4;
                    if (cp < 0x80) out += (char)cp;
                    else if (cp < 0x800) { out += (char)(0xC0 | (cp >> 6)); out += (char)(0x80 | (cp & 0x3F)); }
                    else { out += (char)(0xE0 | (cp >> 12)); out += (char)(0x80 | ((cp >> 6) & 0x3F)); out += (char)(0x80 | (cp & 0x3F)); }
                    break;
                }
                default: out += e;
                }
            } else {
                out += c;
            }
        }
        if (i_ >= s_.size()) fail("unterminated string");
        i_++;
        return out;
    }
};

inline Json read_json_file(const std::string &path) {
    std::ifstream f(path);
    if (!f) throw std::runtime_error("Failed to load config file: " + path);
    std::stringstream ss;
    ss << f.rdbuf();
    const std::string text = ss.str();
    return JsonParser(text).parse();
}

// ------------------------------------------------------------------ OBJ
struct Mesh {
    std::vector<double> V;  // [nv][3]
    std::vector<int> F;     // [nf][3], 0-based
    size_t nv() const { return V.size() / 3; }
    size_t nf() const { return F.size() / 3; }
};

inline Mesh read_obj(const std::string &path) {
    std::ifstream f(path);
    if (!f) throw std::runtime_error("cannot open OBJ file " + path);
    Mesh m;
    std::string line;
    while (std::getline(f, line)) {
        std::istringstream ls(line);
        std::string tag;
        if (!(ls >> tag)) continue;
        if (tag == "v") {
            double x = 0, y = 0, z = 0;
            ls >> x >> y;
            if (!(ls >> z)) z = 0.0;
            m.V.push_back(x);
            m.V.push_back(y);
            m.V.push_back(z);
        } else if (tag == "f") {
            std::vector<int> idx;
            std::string tok;
            while (ls >> tok) {
                const long v = std::strtol(tok.c_str(), nullptr, 10);  // stops at '/'
                if (v == 0) throw std::runtime_error("OBJ: bad face index in " + path);
                idx.push_back(v > 0 ? (int)(v - 1) : (int)((long)m.nv() + v));
            }
            if (idx.size() < 2) throw std::runtime_error("OBJ: face with fewer than two corners in " + path);
            if (idx.size() == 2) idx.push_back(idx[0]);
            for (size_t k = 1; k + 1 < idx.size(); k++) {
                m.F.push_back(idx[0]);
                m.F.push_back(idx[k]);
                m.F.push_back(idx[k + 1]);
            }
        }
    }
    for (int i : m.F)
        if (i < 0 || (size_t)i >= m.nv()) throw std::runtime_error("OBJ: face index out of range in " + path);
    return m;
}

// ------------------------------------------------------------------ winding numbers
// Segment soup (a_i -> b_i): sum of the signed angles subtended at p, over 2 pi.
inline double winding_number_2d(const std::vector<double> &seg, const double p[2]) {
    double w = 0.0;
    const size_t n = seg.size() / 4;
    for (size_t i = 0; i < n; i++) {
        const double ax = seg[4 * i] - p[0], ay = seg[4 * i + 1] - p[1];
        const double bx = seg[4 * i + 2] - p[0], by = seg[4 * i + 3] - p[1];
        w += std::atan2(ax * by - ay * bx, ax * bx + ay * by);
    }
    return w / (2.0 * M_PI);
}

// Triangle soup: sum of the signed solid angles (Van Oosterom & Strackee, IEEE TBME 1983) over
// 4 pi; +1 inside a closed surface whose triangles are counter-clockwise seen from outside.
inline double winding_number_3d(const std::vector<double> &tri, const double p[3]) {
    double w = 0.0;
    const size_t n = tri.size() / 9;
    for (size_t i = 0; i < n; i++) {
        double a[3], b[3], c[3];
        for (int k = 0; k < 3; k++) {
            a[k] = tri[9 * i + k] - p[k];
            b[k] = tri[9 * i + 3 + k] - p[k];
            c[k] = tri[9 * i + 6 + k] - p[k];
        }
        const double la = std::sqrt(a[0] * a[0] + a[1] * a[1] + a[2] * a[2]);
        const double lb = std::sqrt(b[0] * b[0] + b[1] * b[1] + b[2] * b[2]);
        const double lc = std::sqrt(c[0] * c[0] + c[1] * c[1] + c[2] * c[2]);
        const double det = a[0] * (b[1] * c[2] - b[2] * c[1]) - a[1] * (b[0] * c[2] - b[2] * c[0]) +
                           a[2] * (b[0] * c[1] - b[1] * c[0]);
        const double ab = a[0] * b[0] + a[1] * b[1] + a[2] * b[2];
        const double bc = b[0] * c[0] + b[1] * c[1] + b[2] * c[2];
        const double ca = c[0] * a[0] + c[1] * a[1] + c[2] * a[2];
        w += 2.0 * std::atan2(det, la * lb * lc + ab * lc + bc * la + ca * lb);
    }
    return w / (4.0 * M_PI);
}

}  // namespace wobapp
