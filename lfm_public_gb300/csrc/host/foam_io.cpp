// OpenFOAM-format text I/O without OpenFOAM (see foam_io.h).
#include "foam_io.h"

#include <cctype>
#include <cerrno>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <sstream>
#include <sys/stat.h>

namespace lfm {
namespace foam {

// ----------------------------------------------------------------------------
std::string readFile(const std::string& path) {
    std::ifstream in(path, std::ios::binary);
    if (!in) throw FoamError("cannot open file " + path);
    std::ostringstream ss;
    ss << in.rdbuf();
    return ss.str();
}

bool fileExists(const std::string& path) {
    struct stat st;
    return stat(path.c_str(), &st) == 0 && S_ISREG(st.st_mode);
}

// ----------------------------------------------------------------------------
void Tokenizer::skipSpace() {
    const size_t n = buf_.size();
    while (pos_ < n) {
        const char c = buf_[pos_];
        if (c == ' ' || c == '\t' || c == '\n' || c == '\r' || c == '\f' || c == '\v') {
            ++pos_;
        } else if (c == '/' && pos_ + 1 < n && buf_[pos_ + 1] == '/') {
            while (pos_ < n && buf_[pos_] != '\n') ++pos_;
        } else if (c == '/' && pos_ + 1 < n && buf_[pos_ + 1] == '*') {
            const size_t e = buf_.find("*/", pos_ + 2);
            pos_ = (e == std::string::npos) ? n : e + 2;
        } else {
            break;
        }
    }
}

bool Tokenizer::atEnd() {
    if (havePeek_) return peeked_.kind == Token::END;
    skipSpace();
    return pos_ >= buf_.size();
}

static bool isPunct(char c) {
    return c == '(' || c == ')' || c == '{' || c == '}' || c == '[' || c == ']' || c == ';' ||
           c == ',';
}

Token Tokenizer::next() {
    if (havePeek_) {
        havePeek_ = false;
        return peeked_;
    }
    skipSpace();
    Token t;
    const size_t n = buf_.size();
    if (pos_ >= n) return t;
    const char c = buf_[pos_];
    if (isPunct(c)) {
        t.kind = Token::PUNCT;
        t.punct = c;
        t.text = std::string(1, c);
        ++pos_;
        return t;
    }
    if (c == '"') {
        size_t e = pos_ + 1;
        while (e < n && buf_[e] != '"') {
            if (buf_[e] == '\\') ++e;
            ++e;
        }
        t.kind = Token::STRING;
        t.text = buf_.substr(pos_ + 1, e - pos_ - 1);
        pos_ = (e < n) ? e + 1 : n;
        return t;
    }
    // Word or number: run until whitespace or punctuation.
    size_t e = pos_;
    while (e < n) {
        const char d = buf_[e];
        if (d == ' ' || d == '\t' || d == '\n' || d == '\r' || isPunct(d) || d == '"') break;
        if (d == '/' && e + 1 < n && (buf_[e + 1] == '/' || buf_[e + 1] == '*')) break;
        ++e;
    }
    t.text = buf_.substr(pos_, e - pos_);
    pos_ = e;
    // Number?
    const char* s = t.text.c_str();
    char* endp = nullptr;
    errno = 0;
    std::strtod(s, &endp);
    if (endp && *endp == '\0' && endp != s) {
        t.kind = Token::NUMBER;
        t.isInteger = t.text.find_first_of(".eEnN") == std::string::npos;
    } else {
        t.kind = Token::WORD;
    }
    return t;
}

Token Tokenizer::peek() {
    if (!havePeek_) {
        peeked_ = next();
        havePeek_ = true;
    }
    return peeked_;
}

void Tokenizer::expectPunct(char c) {
    Token t = next();
    if (t.kind != Token::PUNCT || t.punct != c)
        throw FoamError(std::string("expected '") + c + "' but found '" + t.text + "'");
}

void Tokenizer::rawBytes(void* dst, size_t n) {
    if (havePeek_) throw FoamError("binary read after peek");
    if (pos_ + n > buf_.size()) throw FoamError("binary payload truncated");
    std::memcpy(dst, buf_.data() + pos_, n);
    pos_ += n;
}

double Tokenizer::readDouble() {
    if (havePeek_) {
        Token t = next();
        return tokenToScalar(t, "list");
    }
    skipSpace();
    const char* s = buf_.c_str() + pos_;
    char* e = nullptr;
    const double v = std::strtod(s, &e);
    if (e == s) throw FoamError("expected a number near offset " + std::to_string(pos_));
    pos_ += (size_t)(e - s);
    return v;
}

long long Tokenizer::readInteger() {
    if (havePeek_) {
        Token t = next();
        return (long long)tokenToScalar(t, "list");
    }
    skipSpace();
    const char* s = buf_.c_str() + pos_;
    char* e = nullptr;
    const long long v = std::strtoll(s, &e, 10);
    if (e == s) throw FoamError("expected an integer near offset " + std::to_string(pos_));
    pos_ += (size_t)(e - s);
    return v;
}

// ----------------------------------------------------------------------------
std::string Entry::text() const {
    std::string s;
    for (size_t i = 0; i < tokens.size(); ++i) {
        if (i) s += ' ';
        s += tokens[i].text;
    }
    return s;
}

const Entry* Dict::find(const std::string& key) const {
    for (size_t i = entries.size(); i-- > 0;)
        if (entries[i].key == key) return &entries[i];
    return nullptr;
}

const Dict* Dict::subDict(const std::string& key) const {
    const Entry* e = find(key);
    return (e && e->isDict()) ? e->dict.get() : nullptr;
}

std::vector<std::string> Dict::toc() const {
    std::vector<std::string> keys;
    for (const Entry& e : entries) {
        bool seen = false;
        for (const std::string& k : keys) seen = seen || (k == e.key);
        if (!seen) keys.push_back(e.key);
    }
    return keys;
}

Dict parseDict(Tokenizer& tk, bool topLevel) {
    Dict d;
    while (true) {
        Token t = tk.next();
        if (t.kind == Token::END) {
            if (!topLevel) throw FoamError("unexpected end of input inside a dictionary");
            break;
        }
        if (t.kind == Token::PUNCT && t.punct == '}') {
            if (topLevel) throw FoamError("unbalanced '}'");
            break;
        }
        if (t.kind == Token::PUNCT && t.punct == ';') continue;
        Entry e;
        e.key = t.text;
        // Directives such as #include / #inputMode: keep as ordinary entries.
        Token v = tk.peek();
        if (v.kind == Token::PUNCT && v.punct == '{') {
            tk.next();
            e.dict = std::make_shared<Dict>(parseDict(tk, false));
            d.entries.push_back(std::move(e));
            continue;
        }
        int depth = 0;
        while (true) {
            Token x = tk.next();
            if (x.kind == Token::END) {
                if (topLevel && depth == 0) break;
                throw FoamError("unterminated entry '" + e.key + "'");
            }
            if (x.kind == Token::PUNCT) {
                if (x.punct == '(' || x.punct == '[' || x.punct == '{') ++depth;
                if (x.punct == ')' || x.punct == ']' || x.punct == '}') --depth;
                if (x.punct == ';' && depth == 0) break;
                if (depth < 0) throw FoamError("unbalanced bracket in entry '" + e.key + "'");
            }
            e.tokens.push_back(x);
        }
        d.entries.push_back(std::move(e));
    }
    return d;
}

Dict parseDictFile(const std::string& path) {
    Tokenizer tk(readFile(path));
    try {
        return parseDict(tk, true);
    } catch (const FoamError& err) {
        throw FoamError(path + ": " + err.what());
    }
}

double tokenToScalar(const Token& t, const std::string& context) {
    if (t.kind != Token::NUMBER) {
        if (t.kind == Token::WORD) {
            // OpenFOAM accepts these spellings for special values.
            if (t.text == "inf" || t.text == "Inf") return INFINITY;
            if (t.text == "-inf" || t.text == "-Inf") return -INFINITY;
            if (t.text == "nan" || t.text == "NaN") return NAN;
        }
        throw FoamError("expected a number for '" + context + "' but found '" + t.text + "'");
    }
    return std::strtod(t.text.c_str(), nullptr);
}

bool wordToBool(const std::string& w, bool* ok) {
    static const char* trues[] = {"true", "yes", "on", "y", "t", "any"};
    static const char* falses[] = {"false", "no", "off", "n", "f", "none"};
    *ok = true;
    for (const char* s : trues)
        if (w == s) return true;
    for (const char* s : falses)
        if (w == s) return false;
    // Integers are accepted as switches as well.
    char* e = nullptr;
    const long v = std::strtol(w.c_str(), &e, 10);
    if (e && *e == '\0' && e != w.c_str()) return v != 0;
    *ok = false;
    return false;
}

// ----------------------------------------------------------------------------
Header readHeader(Tokenizer& tk) {
    Header h;
    Token t = tk.peek();
    if (!(t.kind == Token::WORD && t.text == "FoamFile")) return h;
    tk.next();
    tk.expectPunct('{');
    Dict hd = parseDict(tk, false);
    if (const Entry* e = hd.find("format")) h.format = e->text();
    if (const Entry* e = hd.find("class")) h.cls = e->text();
    if (const Entry* e = hd.find("object")) h.object = e->text();
    if (const Entry* e = hd.find("arch")) {
        const std::string a = e->text();
        if (a.find("label=64") != std::string::npos) h.labelBytes = 8;
        if (a.find("scalar=32") != std::string::npos) h.scalarBytes = 4;
    }
    return h;
}

// Reads the count that starts a list and reports whether the list uses the
// uniform `N{value}` form. Leaves the tokenizer after the count.
static long long readListCount(Tokenizer& tk) {
    Token t = tk.next();
    while (t.kind == Token::WORD) t = tk.next();  // skip "List<scalar>" style prefixes
    if (t.kind != Token::NUMBER || !t.isInteger)
        throw FoamError("expected list size but found '" + t.text + "'");
    return std::strtoll(t.text.c_str(), nullptr, 10);
}

// Binary payload "(" raw ")" for n elements of elemBytes each.
static void readBinaryPayload(Tokenizer& tk, void* dst, size_t bytes) {
    // The '(' follows the count directly (after a newline).
    const std::string& b = tk.buffer();
    size_t p = tk.position();
    while (p < b.size() && b[p] != '(') ++p;
    if (p >= b.size()) throw FoamError("binary list without '('");
    tk.skipTo(p + 1);
    tk.rawBytes(dst, bytes);
    tk.expectPunct(')');
}

static std::vector<int64_t> readLabelListBody(Tokenizer& tk, const Header& h) {
    const long long n = readListCount(tk);
    std::vector<int64_t> out((size_t)n);
    // the uniform form N{value}; looked for in the buffer itself, since a
    // peeked token would consume the '(' that opens a binary payload
    {
        const std::string& b = tk.buffer();
        size_t p = tk.position();
        while (p < b.size() && std::isspace((unsigned char)b[p])) ++p;
        if (p < b.size() && b[p] == '{') {
            tk.expectPunct('{');
            const long long v = tk.readInteger();
            tk.expectPunct('}');
            for (auto& x : out) x = v;
            return out;
        }
    }
    if (h.format == "binary") {
        if (h.labelBytes == 4) {
            std::vector<int32_t> tmp((size_t)n);
            readBinaryPayload(tk, tmp.data(), (size_t)n * 4);
            for (size_t i = 0; i < tmp.size(); ++i) out[i] = tmp[i];
        } else {
            readBinaryPayload(tk, out.data(), (size_t)n * 8);
        }
        return out;
    }
    tk.expectPunct('(');
    for (long long i = 0; i < n; ++i) out[(size_t)i] = tk.readInteger();
    tk.expectPunct(')');
    return out;
}

std::vector<int64_t> readLabelList(const std::string& path) {
    Tokenizer tk(readFile(path));
    Header h = readHeader(tk);
    try {
        return readLabelListBody(tk, h);
    } catch (const FoamError& e) {
        throw FoamError(path + ": " + e.what());
    }
}

std::vector<double> readVectorList(const std::string& path) {
    Tokenizer tk(readFile(path));
    Header h = readHeader(tk);
    const long long n = readListCount(tk);
    std::vector<double> out((size_t)n * 3);
    if (h.format == "binary") {
        if (h.scalarBytes == 8) {
            readBinaryPayload(tk, out.data(), (size_t)n * 24);
        } else {
            std::vector<float> tmp((size_t)n * 3);
            readBinaryPayload(tk, tmp.data(), (size_t)n * 12);
            for (size_t i = 0; i < tmp.size(); ++i) out[i] = tmp[i];
        }
        return out;
    }
    tk.expectPunct('(');
    for (long long i = 0; i < n; ++i) {
        tk.expectPunct('(');
        out[(size_t)(3 * i)] = tk.readDouble();
        out[(size_t)(3 * i + 1)] = tk.readDouble();
        out[(size_t)(3 * i + 2)] = tk.readDouble();
        tk.expectPunct(')');
    }
    tk.expectPunct(')');
    return out;
}

void readFaceList(const std::string& path, std::vector<int64_t>& offsets,
                  std::vector<int64_t>& points) {
    Tokenizer tk(readFile(path));
    Header h = readHeader(tk);
    if (h.cls == "faceCompactList") {
        // Two consecutive label lists: offsets (n+1) then the point labels.
        offsets = readLabelListBody(tk, h);
        points = readLabelListBody(tk, h);
        return;
    }
    const long long n = readListCount(tk);
    offsets.assign(1, 0);
    offsets.reserve((size_t)n + 1);
    points.clear();
    points.reserve((size_t)n * 4);
    tk.expectPunct('(');
    for (long long i = 0; i < n; ++i) {
        const long long m = tk.readInteger();
        tk.expectPunct('(');
        for (long long k = 0; k < m; ++k) points.push_back(tk.readInteger());
        tk.expectPunct(')');
        offsets.push_back((int64_t)points.size());
    }
    tk.expectPunct(')');
}

std::vector<Patch> readBoundary(const std::string& path) {
    Tokenizer tk(readFile(path));
    readHeader(tk);
    const long long n = readListCount(tk);
    tk.expectPunct('(');
    std::vector<Patch> out;
    for (long long i = 0; i < n; ++i) {
        Patch p;
        p.name = tk.next().text;
        tk.expectPunct('{');
        Dict d = parseDict(tk, false);
        if (const Entry* e = d.find("type")) p.type = e->text();
        if (const Entry* e = d.find("nFaces")) p.nFaces = std::strtoll(e->text().c_str(), nullptr, 10);
        if (const Entry* e = d.find("startFace"))
            p.startFace = std::strtoll(e->text().c_str(), nullptr, 10);
        if (const Entry* e = d.find("neighbourPatch")) p.neighbourPatch = e->text();
        if (const Entry* e = d.find("myProcNo")) p.myProcNo = std::atoi(e->text().c_str());
        if (const Entry* e = d.find("neighbProcNo")) p.neighbProcNo = std::atoi(e->text().c_str());
        out.push_back(p);
    }
    tk.expectPunct(')');
    return out;
}

// ----------------------------------------------------------------------------
VolField readVolField(const std::string& path, int64_t nCells, bool isVector) {
    const std::string text = readFile(path);
    Tokenizer tk(text);
    Header h = readHeader(tk);
    VolField f;
    f.isVector = isVector;
    const size_t width = isVector ? 3 : 1;
    f.values.assign((size_t)nCells * width, 0.0);
    bool haveInternal = false;
    while (!tk.atEnd()) {
        Token key = tk.next();
        if (key.kind == Token::PUNCT && key.punct == ';') continue;
        if (key.text == "dimensions") {
            std::string dims;
            Token x = tk.next();
            while (!(x.kind == Token::PUNCT && x.punct == ';')) {
                if (!dims.empty() && !(x.kind == Token::PUNCT && x.punct == ']') &&
                    dims.back() != '[')
                    dims += ' ';
                dims += x.text;
                x = tk.next();
            }
            f.dimensions = dims;
        } else if (key.text == "internalField") {
            Token kind = tk.next();
            if (kind.text == "uniform") {
                if (isVector) {
                    tk.expectPunct('(');
                    double v[3];
                    for (int k = 0; k < 3; ++k) v[k] = tk.readDouble();
                    tk.expectPunct(')');
                    for (int64_t c = 0; c < nCells; ++c)
                        for (int k = 0; k < 3; ++k) f.values[(size_t)(3 * c + k)] = v[k];
                } else {
                    const double v = tk.readDouble();
                    for (int64_t c = 0; c < nCells; ++c) f.values[(size_t)c] = v;
                }
                tk.expectPunct(';');
            } else if (kind.text == "nonuniform") {
                const long long n = readListCount(tk);
                if (n != nCells)
                    throw FoamError(path + ": internalField has " + std::to_string(n) +
                                    " values for " + std::to_string(nCells) + " cells");
                if (h.format == "binary") {
                    readBinaryPayload(tk, f.values.data(), (size_t)n * width * 8);
                } else {
                    tk.expectPunct('(');
                    for (long long c = 0; c < n; ++c) {
                        if (isVector) {
                            tk.expectPunct('(');
                            for (int k = 0; k < 3; ++k) f.values[(size_t)(3 * c + k)] = tk.readDouble();
                            tk.expectPunct(')');
                        } else {
                            f.values[(size_t)c] = tk.readDouble();
                        }
                    }
                    tk.expectPunct(')');
                }
                tk.expectPunct(';');
            } else {
                throw FoamError(path + ": unsupported internalField form '" + kind.text + "'");
            }
            haveInternal = true;
        } else if (key.text == "boundaryField") {
            tk.expectPunct('{');
            const size_t start = tk.position();
            int depth = 1;
            size_t endPos = start;
            while (depth > 0) {
                Token x = tk.next();
                if (x.kind == Token::END) throw FoamError(path + ": unterminated boundaryField");
                if (x.kind == Token::PUNCT && x.punct == '{') ++depth;
                if (x.kind == Token::PUNCT && x.punct == '}') {
                    --depth;
                    if (depth == 0) endPos = tk.position() - 1;
                }
            }
            f.boundaryText = text.substr(start, endPos - start);
        } else {
            // Unknown top-level entry: skip to its ';' (or its closing brace).
            int depth = 0;
            while (true) {
                Token x = tk.next();
                if (x.kind == Token::END) break;
                if (x.kind == Token::PUNCT && (x.punct == '{' || x.punct == '(')) ++depth;
                if (x.kind == Token::PUNCT && (x.punct == '}' || x.punct == ')')) {
                    --depth;
                    if (depth == 0 && x.punct == '}') break;
                }
                if (x.kind == Token::PUNCT && x.punct == ';' && depth == 0) break;
            }
        }
    }
    if (!haveInternal) throw FoamError(path + ": no internalField");
    return f;
}

std::string formatGeneral(double v, int precision) {
    std::ostringstream os;
    os.precision(precision);
    os << v;
    return os.str();
}

void writeVolField(const std::string& path, const VolField& f, const std::string& location,
                   int precision, bool binary) {
    std::ofstream out(path, std::ios::binary);
    if (!out) throw FoamError("cannot write " + path);
    const size_t width = f.isVector ? 3 : 1;
    const size_t n = f.values.size() / width;
    out << "FoamFile\n{\n    version     2.0;\n    format      " << (binary ? "binary" : "ascii")
        << ";\n";
    if (binary) out << "    arch        \"LSB;label=32;scalar=64\";\n";
    out << "    class       " << (f.isVector ? "volVectorField" : "volScalarField") << ";\n"
        << "    location    \"" << location << "\";\n"
        << "    object      " << f.name << ";\n}\n\n";
    out << "dimensions      " << f.dimensions << ";\n\n";
    out << "internalField   nonuniform List<" << (f.isVector ? "vector" : "scalar") << "> \n"
        << n << "\n";
    if (binary) {
        out << "(";
        out.write(reinterpret_cast<const char*>(f.values.data()),
                  (std::streamsize)(f.values.size() * sizeof(double)));
        out << ")\n;\n\n";
    } else {
        out << "(\n";
        char buf[128];
        for (size_t c = 0; c < n; ++c) {
            if (f.isVector) {
                std::snprintf(buf, sizeof(buf), "(%.*g %.*g %.*g)\n", precision, f.values[3 * c],
                              precision, f.values[3 * c + 1], precision, f.values[3 * c + 2]);
            } else {
                std::snprintf(buf, sizeof(buf), "%.*g\n", precision, f.values[c]);
            }
            out << buf;
        }
        out << ")\n;\n\n";
    }
    out << "boundaryField\n{" << f.boundaryText << "}\n";
}

}  // namespace foam
}  // namespace lfm
