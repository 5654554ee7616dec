// Minimal readers for the two text formats on the genome path:
//  - YAML, the subset a variation library uses (read by yaml-cpp in the reference,
//    src/variation_table.cpp:183): block mappings, `|-`/`|` literal blocks, quoted scalars,
//    `{}`, `[a, b]` flow lists, null values, `#` comment lines;
//  - XML, the subset flam3 genomes use (read by pugixml in the reference, src/flame.cpp:161):
//    elements, attributes, comments, declarations, character entities.
#include <cctype>
#include <cstring>

#include "internal.h"

namespace rfk {

namespace {

std::string trim(const std::string& s) {
    size_t b = 0, e = s.size();
    while (b < e && isspace((unsigned char)s[b])) b++;
    while (e > b && isspace((unsigned char)s[e - 1])) e--;
    return s.substr(b, e - b);
}

int indent_of(const std::string& s) {
    int i = 0;
    while (i < (int)s.size() && s[i] == ' ') i++;
    return i;
}

bool is_comment_or_blank(const std::string& s) {
    std::string t = trim(s);
    return t.empty() || t[0] == '#';
}

YNode scalar_node(const std::string& raw) {
    YNode n;
    std::string t = trim(raw);
    if (t.empty()) { n.kind = YNode::Null; return n; }
    if (t == "{}") { n.kind = YNode::Map; return n; }
    if (t.size() >= 2 && t.front() == '[' && t.back() == ']') {
        n.kind = YNode::List;
        std::string inner = t.substr(1, t.size() - 2);
        size_t p = 0;
        while (p <= inner.size()) {
            size_t c = inner.find(',', p);
            if (c == std::string::npos) c = inner.size();
            std::string item = trim(inner.substr(p, c - p));
            if (!item.empty()) n.list.push_back(item);
            p = c + 1;
        }
        return n;
    }
    n.kind = YNode::Scalar;
    if (t.size() >= 2 && (t.front() == '"' || t.front() == '\'') && t.back() == t.front()) {
        std::string body = t.substr(1, t.size() - 2), o;
        if (t.front() == '"') {
            for (size_t i = 0; i < body.size(); i++) {
                if (body[i] == '\\' && i + 1 < body.size()) { o += body[++i]; continue; }
                o += body[i];
            }
        } else {
            for (size_t i = 0; i < body.size(); i++) {
                if (body[i] == '\'' && i + 1 < body.size() && body[i + 1] == '\'') { o += '\''; i++; continue; }
                o += body[i];
            }
        }
        n.text = o;
    } else {
        n.text = t;
    }
    return n;
}

struct YReader {
    std::vector<std::string> lines;
    size_t pos = 0;
    std::string err;

    bool block(int min_indent, YNode& out) {
        out.kind = YNode::Map;
        int ind = -1;
        while (pos < lines.size()) {
            const std::string& raw = lines[pos];
            if (is_comment_or_blank(raw)) { pos++; continue; }
            int i = indent_of(raw);
            if (ind < 0) {
                if (i < min_indent) break;
                ind = i;
            }
            if (i < ind) break;
            if (i > ind) { err = "unexpected indentation at line " + std::to_string(pos + 1); return false; }
            std::string body = trim(raw);
            size_t colon = body.find(':');
            if (colon == std::string::npos) { err = "expected `key: value` at line " + std::to_string(pos + 1); return false; }
            std::string key = trim(body.substr(0, colon));
            std::string rest = trim(body.substr(colon + 1));
            pos++;
            YNode val;
            if (rest == "|-" || rest == "|") {
                std::vector<std::string> got;
                int bind = -1;
                while (pos < lines.size()) {
                    const std::string& r2 = lines[pos];
                    if (trim(r2).empty()) { got.push_back(""); pos++; continue; }
                    int i2 = indent_of(r2);
                    if (bind < 0) {
                        if (i2 <= ind) break;
                        bind = i2;
                    }
                    if (i2 < bind) break;
                    got.push_back(r2.substr(bind));
                    pos++;
                }
                while (!got.empty() && got.back().empty()) got.pop_back();
                val.kind = YNode::Scalar;
                for (size_t k = 0; k < got.size(); k++) {
                    if (k) val.text += '\n';
                    val.text += got[k];
                }
                if (rest == "|") val.text += '\n';
            } else if (rest.empty()) {
                size_t save = pos;
                while (pos < lines.size() && is_comment_or_blank(lines[pos])) pos++;
                if (pos < lines.size() && indent_of(lines[pos]) > ind) {
                    if (!block(ind + 1, val)) return false;
                } else {
                    pos = save;
                    val.kind = YNode::Null;
                }
            } else {
                val = scalar_node(rest);
            }
            out.map.emplace_back(key, std::move(val));
        }
        return true;
    }
};

std::string xml_unescape(std::string s) {
    if (s.find('&') == std::string::npos) return s;  // nothing escaped: the text itself
    std::string o;
    for (size_t i = 0; i < s.size(); i++) {
        if (s[i] == '&') {
            size_t e = s.find(';', i);
            if (e != std::string::npos && e - i < 10) {
                std::string ent = s.substr(i + 1, e - i - 1);
                if (ent == "amp") { o += '&'; i = e; continue; }
                if (ent == "lt") { o += '<'; i = e; continue; }
                if (ent == "gt") { o += '>'; i = e; continue; }
                if (ent == "quot") { o += '"'; i = e; continue; }
                if (ent == "apos") { o += '\''; i = e; continue; }
                if (!ent.empty() && ent[0] == '#') {
                    long v = (ent.size() > 1 && (ent[1] == 'x' || ent[1] == 'X')) ? strtol(ent.c_str() + 2, nullptr, 16)
                                                                                  : strtol(ent.c_str() + 1, nullptr, 10);
                    if (v > 0 && v < 128) { o += (char)v; i = e; continue; }
                }
            }
        }
        o += s[i];
    }
    return o;
}

// XML whitespace (the S production: space, tab, CR, LF)
inline bool xml_space(char c) { return c == ' ' || c == '\t' || c == '\n' || c == '\r'; }

struct XReader {
    const std::string& s;
    size_t i = 0;
    std::string err;
    explicit XReader(const std::string& t) : s(t) {}

    void ws() { while (i < s.size() && xml_space(s[i])) i++; }
    // skips comments, declarations, processing instructions; stops at '<' of an element or end tag
    bool misc(std::string* text) {
        for (;;) {
            size_t b = i;
            const void* lt = i < s.size() ? memchr(s.data() + i, '<', s.size() - i) : nullptr;
            i = lt ? (size_t)(static_cast<const char*>(lt) - s.data()) : s.size();
            if (text) text->append(s, b, i - b);
            if (i >= s.size()) return false;
            if (s.compare(i, 4, "<!--") == 0) {
                size_t e = s.find("-->", i + 4);
                if (e == std::string::npos) { err = "unterminated comment"; return false; }
                i = e + 3; continue;
            }
            if (s.compare(i, 9, "<![CDATA[") == 0) {
                size_t e = s.find("]]>", i + 9);
                if (e == std::string::npos) { err = "unterminated CDATA"; return false; }
                if (text) *text += s.substr(i + 9, e - i - 9);
                i = e + 3; continue;
            }
            if (s.compare(i, 2, "<?") == 0) {
                size_t e = s.find("?>", i + 2);
                if (e == std::string::npos) { err = "unterminated declaration"; return false; }
                i = e + 2; continue;
            }
            if (s.compare(i, 2, "<!") == 0) {
                size_t e = s.find('>', i + 2);
                if (e == std::string::npos) { err = "unterminated declaration"; return false; }
                i = e + 1; continue;
            }
            return true;
        }
    }
    bool element(XNode& out, int depth) {
        if (depth > 64) { err = "nesting too deep"; return false; }
        i++;  // '<'
        size_t b = i;
        while (i < s.size() && !xml_space(s[i]) && s[i] != '>' && s[i] != '/') i++;
        out.name.assign(s, b, i - b);
        if (out.name.empty()) { err = "empty element name"; return false; }
        for (;;) {
            ws();
            if (i >= s.size()) { err = "end of input inside <" + out.name + ">"; return false; }
            if (s[i] == '/') {
                if (i + 1 < s.size() && s[i + 1] == '>') { i += 2; return true; }
                err = "stray '/' in <" + out.name + ">"; return false;
            }
            if (s[i] == '>') { i++; break; }
            size_t ab = i;
            while (i < s.size() && s[i] != '=' && !xml_space(s[i]) && s[i] != '>') i++;
            std::string an = s.substr(ab, i - ab);
            ws();
            if (i >= s.size() || s[i] != '=') { err = "attribute `" + an + "` without a value"; return false; }
            i++;
            ws();
            if (i >= s.size() || (s[i] != '"' && s[i] != '\'')) { err = "unquoted attribute `" + an + "`"; return false; }
            char q = s[i++];
            size_t vb = i;
            const void* qe = i < s.size() ? memchr(s.data() + i, q, s.size() - i) : nullptr;
            i = qe ? (size_t)(static_cast<const char*>(qe) - s.data()) : s.size();
            if (i >= s.size()) { err = "unterminated attribute `" + an + "`"; return false; }
            out.attrs.emplace_back(an, xml_unescape(s.substr(vb, i - vb)));
            i++;
        }
        for (;;) {
            if (!misc(&out.text)) { if (err.empty()) err = "end of input inside <" + out.name + ">"; return false; }
            if (s.compare(i, 2, "</") == 0) {
                size_t e = s.find('>', i);
                if (e == std::string::npos) { err = "unterminated end tag"; return false; }
                std::string nm = trim(s.substr(i + 2, e - i - 2));
                if (nm != out.name) { err = "mismatched </" + nm + "> for <" + out.name + ">"; return false; }
                i = e + 1;
                out.text = xml_unescape(std::move(out.text));
                return true;
            }
            XNode k;
            if (!element(k, depth + 1)) return false;
            out.kids.push_back(std::move(k));
        }
    }
};

}  // namespace

// FNV-1a over a variation's src and result text with whitespace left out (so re-indented or
// re-wrapped YAML hashes alike), the two parts separated by 0x1f.
uint64_t snippet_hash(const std::string& src, const std::string& result) {
    uint64_t h = 1469598103934665603ull;
    auto feed = [&](const std::string& s) {
        for (unsigned char ch : s) {
            if (std::isspace(ch)) continue;
            h ^= ch;
            h *= 1099511628211ull;
        }
    };
    feed(src);
    h ^= 0x1f;
    h *= 1099511628211ull;
    feed(result);
    return h;
}

bool parse_yaml(const std::string& text, YNode& out, std::string& err) {
    YReader r;
    size_t p = 0;
    while (p <= text.size()) {
        size_t e = text.find('\n', p);
        if (e == std::string::npos) e = text.size();
        std::string ln = text.substr(p, e - p);
        if (!ln.empty() && ln.back() == '\r') ln.pop_back();
        if (ln.find('\t') != std::string::npos && trim(ln).size() && ln.find_first_not_of(" \t") > ln.find('\t')) {
            err = "tab indentation at line " + std::to_string(r.lines.size() + 1);
            return false;
        }
        r.lines.push_back(ln);
        p = e + 1;
    }
    if (!r.block(0, out)) { err = r.err; return false; }
    if (r.pos < r.lines.size()) {
        // anything left is dedented garbage
        for (size_t k = r.pos; k < r.lines.size(); k++)
            if (!is_comment_or_blank(r.lines[k])) { err = "unexpected content at line " + std::to_string(k + 1); return false; }
    }
    return true;
}

bool parse_xml(const std::string& text, std::vector<XNode>& roots, std::string& err) {
    XReader r(text);
    for (;;) {
        if (!r.misc(nullptr)) {
            if (!r.err.empty()) { err = r.err; return false; }
            break;
        }
        if (text.compare(r.i, 2, "</") == 0) { err = "unexpected end tag"; return false; }
        XNode n;
        if (!r.element(n, 0)) { err = r.err; return false; }
        roots.push_back(std::move(n));
    }
    if (roots.empty()) { err = "no XML element"; return false; }
    return true;
}

}  // namespace rfk
