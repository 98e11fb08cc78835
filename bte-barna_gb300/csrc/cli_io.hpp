// cli_io.hpp - input helpers shared by the drop-in executables: a minimal
// XML reader (elements, attributes, text; skips <? ?> and <!-- -->), path
// resolution relative to the input file, and the BTEMODE1 mode-table file
// (the engine's stand-in for the reference's HDF5 databases).
#pragma once

#include <cctype>
#include <cstdint>
#include <cstdio>
#include <fstream>
#include <map>
#include <memory>
#include <sstream>
#include <stdexcept>
#include <string>
#include <vector>

namespace bte_cli {

struct Node {
    std::string name, text;
    std::map<std::string, std::string> attr;
    std::vector<std::unique_ptr<Node>> kids;
    const Node* child(const std::string& n) const {
        for (auto& k : kids)
            if (k->name == n) return k.get();
        return nullptr;
    }
    std::string get(const std::string& a) const {
        auto it = attr.find(a);
        if (it == attr.end()) throw std::runtime_error("missing attribute " + a + " in <" + name + ">");
        return it->second;
    }
    bool has(const std::string& a) const { return attr.count(a) != 0; }
};

// Minimal XML reader: elements, attributes, text; skips <? ?>, <!-- -->.
struct XmlReader {
    std::string s;
    std::size_t i = 0;
    void ws() {
        while (i < s.size() && std::isspace((unsigned char)s[i])) ++i;
    }
    void skip_misc() {
        for (;;) {
            ws();
            if (s.compare(i, 4, "<!--") == 0) {
                std::size_t e = s.find("-->", i);
                if (e == std::string::npos) throw std::runtime_error("unterminated comment");
                i = e + 3;
            } else if (s.compare(i, 2, "<?") == 0) {
                std::size_t e = s.find("?>", i);
                if (e == std::string::npos) throw std::runtime_error("unterminated declaration");
                i = e + 2;
            } else {
                return;
            }
        }
    }
    std::string name() {
        std::size_t b = i;
        while (i < s.size() && (std::isalnum((unsigned char)s[i]) || s[i] == '_' || s[i] == '-' || s[i] == ':' || s[i] == '.')) ++i;
        if (b == i) throw std::runtime_error("bad XML name");
        return s.substr(b, i - b);
    }
    std::unique_ptr<Node> element() {
        skip_misc();
        if (i >= s.size() || s[i] != '<') throw std::runtime_error("expected an element");
        ++i;
        auto n = std::make_unique<Node>();
        n->name = name();
        for (;;) {
            ws();
            if (s.compare(i, 2, "/>") == 0) {
                i += 2;
                return n;
            }
            if (s[i] == '>') {
                ++i;
                break;
            }
            std::string a = name();
            ws();
            if (s[i] != '=') throw std::runtime_error("expected = in attribute");
            ++i;
            ws();
            char q = s[i++];
            std::size_t e = s.find(q, i);
            if (e == std::string::npos) throw std::runtime_error("unterminated attribute");
            n->attr[a] = s.substr(i, e - i);
            i = e + 1;
        }
        for (;;) {
            std::size_t b = i;
            while (i < s.size() && s[i] != '<') ++i;
            n->text += s.substr(b, i - b);
            if (i >= s.size()) throw std::runtime_error("unterminated element " + n->name);
            if (s.compare(i, 4, "<!--") == 0) {
                skip_misc();
                continue;
            }
            if (s.compare(i, 2, "</") == 0) {
                i += 2;
                std::string e = name();
                if (e != n->name) throw std::runtime_error("mismatched </" + e + ">");
                ws();
                ++i;  // '>'
                return n;
            }
            n->kids.push_back(element());
        }
    }
};

inline std::unique_ptr<Node> read_xml(const std::string& path) {
    std::ifstream f(path);
    if (!f) throw std::runtime_error("cannot open " + path);
    std::stringstream ss;
    ss << f.rdbuf();
    XmlReader r;
    r.s = ss.str();
    return r.element();
}

inline std::string dir_of(const std::string& p) {
    std::size_t k = p.find_last_of('/');
    return k == std::string::npos ? std::string() : p.substr(0, k + 1);
}

inline std::string resolve(const std::string& base, const std::string& f) {
    if (!f.empty() && f[0] == '/') return f;
    std::ifstream t(f);
    if (t) return f;
    return base + f;
}

struct ModesFile {
    int32_t head[5];
    double V, c, dq[9];
    std::vector<double> omega, vg, w;
};

inline ModesFile read_modes(const std::string& path) {
    std::ifstream f(path, std::ios::binary);
    if (!f) throw std::runtime_error("cannot open database " + path);
    char magic[8];
    f.read(magic, 8);
    if (std::string(magic, 8) != "BTEMODE1")
        throw std::runtime_error(path + " is not a BTEMODE1 mode table (HDF5 databases need libhdf5)");
    ModesFile m;
    f.read(reinterpret_cast<char*>(m.head), sizeof m.head);
    f.read(reinterpret_cast<char*>(&m.V), 8);
    f.read(reinterpret_cast<char*>(&m.c), 8);
    f.read(reinterpret_cast<char*>(m.dq), sizeof m.dq);
    const std::size_t n = std::size_t(m.head[0]) * std::size_t(m.head[1]);
    m.omega.resize(n);
    m.vg.resize(3 * n);
    m.w.resize(n);
    f.read(reinterpret_cast<char*>(m.omega.data()), std::streamsize(n * 8));
    f.read(reinterpret_cast<char*>(m.vg.data()), std::streamsize(3 * n * 8));
    f.read(reinterpret_cast<char*>(m.w.data()), std::streamsize(n * 8));
    if (!f) throw std::runtime_error("truncated mode table " + path);
    return m;
}

inline std::string fmt_g(double x) {
    char b[64];
    std::snprintf(b, sizeof b, "%g", x);
    return b;
}

}  // namespace bte_cli
