// CDictReaderOF without OpenFOAM: reads <dictDirectory>/<dictName> relative to
// the working directory. Same class as the reference's api/dictReaderOF.h:9-70.
#ifndef LFM_DICT_READER_OF_H
#define LFM_DICT_READER_OF_H

#include <string>
#include <vector>

#include "dictReader.h"

class CDictReaderOF : public IDictReader {
public:
    CDictReaderOF(std::string dictName, std::string dictDirectory);
    virtual ~CDictReaderOF();

    virtual std::string readDictWord(std::string paramName, std::vector<std::string> subDictList,
                                     const std::string sDefault = "", const bool bAllowDefault = false);
    virtual std::string readDictWord(std::string paramName, std::string subDict = "",
                                     const std::string sDefault = "", const bool bAllowDefault = false) {
        return readDictWord(paramName, extractSubDictList(subDict), sDefault, bAllowDefault);
    }

    virtual std::string readDictFilename(std::string paramName, std::vector<std::string> subDictList,
                                         const std::string sDefault = "", const bool bAllowDefault = false);
    virtual std::string readDictFilename(std::string paramName, std::string subDict = "",
                                         const std::string sDefault = "", const bool bAllowDefault = false) {
        return readDictFilename(paramName, extractSubDictList(subDict), sDefault, bAllowDefault);
    }

    virtual bool readDictBool(std::string paramName, std::vector<std::string> subDictList,
                              const bool bDefault = true, const bool bAllowDefault = false);
    virtual bool readDictBool(std::string paramName, std::string subDict = "", const bool bDefault = true,
                              const bool bAllowDefault = false) {
        return readDictBool(paramName, extractSubDictList(subDict), bDefault, bAllowDefault);
    }

    virtual double readDictScalar(std::string paramName, std::vector<std::string> subDictList,
                                  const double dDefault = 0, const bool bAllowDefault = false);
    virtual double readDictScalar(std::string paramName, std::string subDict = "", const double dDefault = 0,
                                  const bool bAllowDefault = false) {
        return readDictScalar(paramName, extractSubDictList(subDict), dDefault, bAllowDefault);
    }

    virtual std::string readDictString(std::string paramName, std::vector<std::string> subDictList,
                                       const std::string sDefault = "", const bool bAllowDefault = false);
    virtual std::string readDictString(std::string paramName, std::string subDict = "",
                                       const std::string sDefault = "", const bool bAllowDefault = false) {
        return readDictString(paramName, extractSubDictList(subDict), sDefault, bAllowDefault);
    }

    virtual std::vector<double> readDictVector(std::string paramName, std::vector<std::string> subDictList);
    virtual std::vector<double> readDictVector(std::string paramName, std::string subDict = "") {
        return readDictVector(paramName, extractSubDictList(subDict));
    }

    virtual std::vector<std::string> getKeyList(std::vector<std::string> subDictList) {
        return getKeyOrDictList(true, subDictList);
    }
    virtual std::vector<std::string> getKeyList(std::string subDict = "") { return getKeyOrDictList(true, subDict); }

    virtual std::vector<std::string> getDictList(std::vector<std::string> subDictList) {
        return getKeyOrDictList(false, subDictList);
    }
    virtual std::vector<std::string> getDictList(std::string subDict = "") { return getKeyOrDictList(false, subDict); }

protected:
    std::vector<std::string> extractSubDictList(std::string subDict);
    const void* getDict(std::vector<std::string> subDictList);
    const void* getDict(std::string subDict) { return getDict(extractSubDictList(subDict)); }
    std::vector<std::string> getKeyOrDictList(const bool bKey, std::vector<std::string> subDictList);
    std::vector<std::string> getKeyOrDictList(const bool bKey, std::string subDict = "") {
        return getKeyOrDictList(bKey, extractSubDictList(subDict));
    }

    void* m_pIODict;
};

#endif
