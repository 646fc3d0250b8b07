// IDictReader: typed lookups in an OpenFOAM-format dictionary, with
// sub-dictionary paths "a/b/c". Same interface as the reference's
// api/dictReader.h:7-44.
#ifndef LFM_DICT_READER_H
#define LFM_DICT_READER_H

#include <string>
#include <vector>

class IDictReader {
public:
    virtual ~IDictReader() {}

    virtual std::string readDictWord(std::string paramName, std::vector<std::string> subDictList,
                                     const std::string sDefault = "", const bool bAllowDefault = false) = 0;
    virtual std::string readDictWord(std::string paramName, std::string subDict = "",
                                     const std::string sDefault = "", const bool bAllowDefault = false) = 0;

    virtual std::string readDictFilename(std::string paramName, std::vector<std::string> subDictList,
                                         const std::string sDefault = "", const bool bAllowDefault = false) = 0;
    virtual std::string readDictFilename(std::string paramName, std::string subDict = "",
                                         const std::string sDefault = "", const bool bAllowDefault = false) = 0;

    virtual bool readDictBool(std::string paramName, std::vector<std::string> subDictList,
                              const bool bDefault = true, const bool bAllowDefault = false) = 0;
    virtual bool readDictBool(std::string paramName, std::string subDict = "", const bool bDefault = true,
                              const bool bAllowDefault = false) = 0;

    virtual double readDictScalar(std::string paramName, std::vector<std::string> subDictList,
                                  const double dDefault = 0, const bool bAllowDefault = false) = 0;
    virtual double readDictScalar(std::string paramName, std::string subDict = "", const double dDefault = 0,
                                  const bool bAllowDefault = false) = 0;

    virtual std::string readDictString(std::string paramName, std::vector<std::string> subDictList,
                                       const std::string sDefault = "", const bool bAllowDefault = false) = 0;
    virtual std::string readDictString(std::string paramName, std::string subDict = "",
                                       const std::string sDefault = "", const bool bAllowDefault = false) = 0;

    virtual std::vector<double> readDictVector(std::string paramName, std::vector<std::string> subDictList) = 0;
    virtual std::vector<double> readDictVector(std::string paramName, std::string subDict = "") = 0;

    virtual std::vector<std::string> getKeyList(std::vector<std::string> subDictList) = 0;
    virtual std::vector<std::string> getKeyList(std::string subDict = "") = 0;

    virtual std::vector<std::string> getDictList(std::vector<std::string> subDictList) = 0;
    virtual std::vector<std::string> getDictList(std::string subDict = "") = 0;
};

#endif
