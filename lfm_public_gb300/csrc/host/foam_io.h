// OpenFOAM-format text I/O without OpenFOAM.
//
// The reference reads its case through three OpenFOAM plugins
// (dictReaderOF/dictReaderOF.cpp:19-35 IOdictionary, polyMeshReaderOF/
// polyMeshReaderOF.cpp:15-68 fvMesh, runTimeManagerOF/runTimeManagerOF.cpp:5-13
// Foam::Time). This module restates the parts of the OpenFOAM file grammar that
// those plugins consume: the FoamFile header, nested dictionaries with
// `key value;` entries, comments, labelList / vectorField / faceList blocks in
// ascii and binary format, and the volScalarField / volVectorField layout.
#pragma once

#include <cstdint>
#include <map>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

namespace lfm {
namespace foam {

// Errors in case files surface as this exception; the plugin layer turns it
// into the reference's behaviour (a fatal message and a non-zero exit).
struct FoamError : public std::runtime_error {
    explicit FoamError(const std::string& m) : std::runtime_error(m) {}
};

struct Token {
    enum Kind { WORD, NUMBER, STRING, PUNCT, END };
    Kind kind = END;
    std::string text;  // raw text (words, numbers, strings without quotes)
    char punct = 0;    // one of ( ) { } [ ] ; ,
    bool isInteger = false;
};

// Tokenizer over an in-memory buffer. Handles // and /* */ comments, quoted
// strings and the punctuation OpenFOAM uses. Binary list payloads are read
// through rawBytes() at the current position.
class Tokenizer {
public:
    explicit Tokenizer(std::string buffer) : buf_(std::move(buffer)) {}
    Token next();
    Token peek();
    void expectPunct(char c);
    size_t position() const { return pos_; }
    void rawBytes(void* dst, size_t n);   // copies n bytes at the cursor
    bool atEnd();
    const std::string& buffer() const { return buf_; }
    void skipTo(size_t p) { pos_ = p; havePeek_ = false; }
    // Fast paths for large ascii lists.
    double readDouble();
    long long readInteger();
private:
    void skipSpace();
    std::string buf_;
    size_t pos_ = 0;
    bool havePeek_ = false;
    Token peeked_;
};

// A dictionary entry is either a sub-dictionary or a token stream ending at ';'.
struct Dict;
struct Entry {
    std::string key;
    std::shared_ptr<Dict> dict;    // non-null for sub-dictionaries
    std::vector<Token> tokens;     // value tokens otherwise
    bool isDict() const { return dict != nullptr; }
    std::string text() const;      // tokens joined by single spaces
};

struct Dict {
    std::vector<Entry> entries;
    const Entry* find(const std::string& key) const;  // last definition wins
    const Dict* subDict(const std::string& key) const;
    std::vector<std::string> toc() const;
};

// Parses `key value;` / `key { ... }` sequences until the closing brace (or end
// of input when topLevel). The FoamFile header is parsed like any other entry.
Dict parseDict(Tokenizer& tk, bool topLevel);
Dict parseDictFile(const std::string& path);

std::string readFile(const std::string& path);
bool fileExists(const std::string& path);

// Scalar / bool / word conversions with OpenFOAM's spellings.
double tokenToScalar(const Token& t, const std::string& context);
bool wordToBool(const std::string& w, bool* ok);

// The FoamFile header of a data file and the position where the payload starts.
struct Header {
    std::string format = "ascii";   // ascii | binary
    std::string cls;
    std::string object;
    int labelBytes = 4;
    int scalarBytes = 8;
};
Header readHeader(Tokenizer& tk);

// List readers for polyMesh files (ascii and binary payloads).
std::vector<int64_t> readLabelList(const std::string& path);
std::vector<double> readVectorList(const std::string& path);            // xyz triples
void readFaceList(const std::string& path, std::vector<int64_t>& offsets,
                  std::vector<int64_t>& points);                        // CSR
struct Patch {
    std::string name, type;
    int64_t nFaces = 0, startFace = 0;
    std::string neighbourPatch;     // cyclic partner name
    int myProcNo = -1, neighbProcNo = -1;
};
std::vector<Patch> readBoundary(const std::string& path);

// Volume fields: the internal values and the boundaryField block kept as text so
// that a field read from disk is written back with its own patch entries.
struct VolField {
    std::string name;
    bool isVector = false;
    std::vector<double> values;          // n or 3n values
    std::string dimensions = "[0 0 0 0 0 0 0]";
    std::string boundaryText;            // contents between boundaryField braces
};
VolField readVolField(const std::string& path, int64_t nCells, bool isVector);

// Writers. `precision` is the controlDict writePrecision.
void writeVolField(const std::string& path, const VolField& f, const std::string& location,
                   int precision, bool binary);
std::string formatGeneral(double v, int precision);

}  // namespace foam
}  // namespace lfm
