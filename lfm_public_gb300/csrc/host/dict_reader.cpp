// CDictReaderOF without OpenFOAM.
//
// Follows dictReaderOF/dictReaderOF.cpp: the dictionary is
// <dictDirectory>/<dictName> under the working directory (:19-35); sub-dictionary
// paths "a/b" descend with optionalSubDict semantics, i.e. a missing level
// leaves the lookup at the current level (:132-139); lookups with a default use
// getOrDefault (:148-153), lookups without one are fatal when the key is absent.
// A fatal error prints an OpenFOAM-style message and throws lfm::foam::FoamError.
#include "dictReaderOF.h"

#include <cstdio>
#include <iostream>

#include "foam_io.h"

using lfm::foam::Dict;
using lfm::foam::Entry;
using lfm::foam::FoamError;

namespace {
struct DictHolder {
    std::string path;
    Dict dict;
};

[[noreturn]] void fatal(const DictHolder* h, const std::string& msg) {
    std::cerr << "\n--> FOAM FATAL IO ERROR:\n" << msg << "\n\nfile: " << h->path << "\n" << std::endl;
    throw FoamError(h->path + ": " + msg);
}

const Entry* lookup(const DictHolder* h, const Dict* d, const std::string& key, bool mandatory) {
    const Entry* e = d->find(key);
    if (!e && mandatory) fatal(h, "Entry '" + key + "' not found in dictionary");
    return e;
}
}  // namespace

CDictReaderOF::CDictReaderOF(std::string dictName, std::string dictDirectory) {
    DictHolder* h = new DictHolder;
    h->path = dictDirectory.empty() ? dictName : dictDirectory + "/" + dictName;
    try {
        h->dict = lfm::foam::parseDictFile(h->path);
    } catch (const FoamError& err) {
        std::cerr << "\n--> FOAM FATAL ERROR:\ncannot read dictionary " << h->path << ": " << err.what()
                  << std::endl;
        delete h;
        throw;
    }
    m_pIODict = h;
}

CDictReaderOF::~CDictReaderOF() {
    delete static_cast<DictHolder*>(m_pIODict);
    m_pIODict = nullptr;
}

std::vector<std::string> CDictReaderOF::extractSubDictList(std::string subDict) {
    std::vector<std::string> out;
    if (subDict.empty()) return out;
    size_t start = 0;
    while (true) {
        const size_t slash = subDict.find('/', start);
        if (slash == std::string::npos) {
            out.push_back(subDict.substr(start));
            break;
        }
        out.push_back(subDict.substr(start, slash - start));
        start = slash + 1;
    }
    return out;
}

const void* CDictReaderOF::getDict(std::vector<std::string> subDictList) {
    const DictHolder* h = static_cast<const DictHolder*>(m_pIODict);
    const Dict* d = &h->dict;
    for (const std::string& name : subDictList) {
        const Dict* sub = d->subDict(name);
        if (sub) d = sub;  // optionalSubDict: stay at this level when missing
    }
    return d;
}

std::vector<std::string> CDictReaderOF::getKeyOrDictList(const bool bKey, std::vector<std::string> subDictList) {
    const Dict* d = static_cast<const Dict*>(getDict(subDictList));
    std::vector<std::string> out;
    for (const std::string& key : d->toc()) {
        if (key == "FoamFile") continue;
        const bool isDict = d->find(key)->isDict();
        if (isDict != bKey) out.push_back(key);
    }
    return out;
}

static std::string entryWord(const DictHolder* h, const Entry* e) {
    if (e->isDict() || e->tokens.empty()) fatal(h, "Entry '" + e->key + "' is not a word");
    return e->tokens[0].text;
}

std::string CDictReaderOF::readDictWord(std::string paramName, std::vector<std::string> subDictList,
                                        const std::string sDefault, const bool bAllowDefault) {
    const DictHolder* h = static_cast<const DictHolder*>(m_pIODict);
    const Entry* e = lookup(h, static_cast<const Dict*>(getDict(subDictList)), paramName, !bAllowDefault);
    return e ? entryWord(h, e) : sDefault;
}

std::string CDictReaderOF::readDictFilename(std::string paramName, std::vector<std::string> subDictList,
                                            const std::string sDefault, const bool bAllowDefault) {
    return readDictWord(paramName, subDictList, sDefault, bAllowDefault);
}

bool CDictReaderOF::readDictBool(std::string paramName, std::vector<std::string> subDictList, const bool bDefault,
                                 const bool bAllowDefault) {
    const DictHolder* h = static_cast<const DictHolder*>(m_pIODict);
    const Entry* e = lookup(h, static_cast<const Dict*>(getDict(subDictList)), paramName, !bAllowDefault);
    if (!e) return bDefault;
    bool ok = false;
    const bool v = lfm::foam::wordToBool(entryWord(h, e), &ok);
    if (!ok) fatal(h, "Entry '" + paramName + "' is not a bool: " + e->text());
    return v;
}

double CDictReaderOF::readDictScalar(std::string paramName, std::vector<std::string> subDictList,
                                     const double dDefault, const bool bAllowDefault) {
    const DictHolder* h = static_cast<const DictHolder*>(m_pIODict);
    const Entry* e = lookup(h, static_cast<const Dict*>(getDict(subDictList)), paramName, !bAllowDefault);
    if (!e) return dDefault;
    if (e->isDict() || e->tokens.empty()) fatal(h, "Entry '" + paramName + "' is not a scalar");
    try {
        return lfm::foam::tokenToScalar(e->tokens[0], paramName);
    } catch (const FoamError& err) {
        fatal(h, err.what());
    }
}

std::string CDictReaderOF::readDictString(std::string paramName, std::vector<std::string> subDictList,
                                          const std::string /*sDefault*/, const bool /*bAllowDefault*/) {
    // The reference always looks the key up (dictReaderOF.cpp:77-81), so a
    // missing key is fatal whatever the default arguments say.
    const DictHolder* h = static_cast<const DictHolder*>(m_pIODict);
    const Entry* e = lookup(h, static_cast<const Dict*>(getDict(subDictList)), paramName, true);
    return e->text();
}

std::vector<double> CDictReaderOF::readDictVector(std::string paramName, std::vector<std::string> subDictList) {
    const DictHolder* h = static_cast<const DictHolder*>(m_pIODict);
    const Entry* e = lookup(h, static_cast<const Dict*>(getDict(subDictList)), paramName, true);
    std::vector<double> out;
    for (const lfm::foam::Token& t : e->tokens)
        if (t.kind == lfm::foam::Token::NUMBER) out.push_back(lfm::foam::tokenToScalar(t, paramName));
    if (out.size() != 3) fatal(h, "Entry '" + paramName + "' is not a vector: " + e->text());
    return out;
}
