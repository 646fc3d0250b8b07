// CInputReader: case parameters from the OpenFOAM dictionaries and the command
// line. Same public members and lookups as the reference's api/inputReader.h:
// 11-88 and src/inputReader.cpp:7-196; readCase() additionally reads a case
// rooted at a directory other than the working directory.
#ifndef LFM_INPUT_READER_H
#define LFM_INPUT_READER_H

#include <string>

class CInputReader {
public:
    CInputReader() {}

    // Reads system/, constant/ of the working directory, then the flags
    // -h/--help, -p/--parallel, -c/--comm_type. Returns false when the run
    // must stop (help requested or a bad flag), as the reference does.
    bool initialize(int argc, char* argv[]);

    // Reads the dictionaries of the case rooted at `root`.
    void readCase(const std::string& root);

protected:
    static void showUsage(char* argv[]);
    bool parseHaloCommType(const char* sCommType);
    bool readRuntimeArgs(int argc, char* argv[]);

public:
    bool m_bParallel = false;

    // system/controlDict
    int m_nCommType = 2;
    int m_nHaloCommType = 1;
    bool m_bIsDoublePrecision = true;
    bool m_bHaveProbes = false;
    bool m_bHaveSampling = false;
    bool m_bHaveAverage = false;
    bool m_bHaveForces = false;
    bool m_bHaveResidual = false;
    int m_nSaveForcesSteps = 1;
    int m_nPrintInfoFrequency = 1;
    bool m_bSaveResiduals = false;
    bool m_bSaveBlendFactor = false;
    bool m_bSaveRank = false;
    bool m_bSaveCellOrder = false;
    double m_dCFLMax = 1;
    double m_tStartAverage = 0;

    // system/fvSchemes
    int m_nSolver = 0;
    int m_nDimension = 2;
    int m_nRkStepCount = 5;
    bool m_bMinmodInterpolation = false;
    bool m_bConstantTimeStep = true;

    // constant/spongeDict
    double m_dPInf = 0;
    double m_dTInf = 0;
    double m_dUInf[3] = {0, 0, 0};
    double m_dLs = 0;
    double m_dMach = 0;
    double m_dK = 0;

    // constant/thermophysicalProperties
    double m_dCp = 0;
    double m_dMolWeight = 0;
    double m_dMu0 = 0;
    double m_dPrandtl = 0;

    // constant/turbulenceProperties
    bool m_bisLaminar = true;
};

#endif
