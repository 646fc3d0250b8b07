// CInputReader for the product: the same dictionary lookups, defaults and
// command-line flags as the reference's src/inputReader.cpp:7-196, over the
// OpenFOAM-free CDictReaderOF.
#include "inputReader.h"

#include <cstdio>
#include <cstring>
#include <getopt.h>
#include <iostream>

#include "dictReaderOF.h"

void CInputReader::readCase(const std::string& root) {
    const std::string sys = root + "/system", cst = root + "/constant";
    CDictReaderOF controlDict("controlDict", sys);
    m_nCommType = (int)controlDict.readDictScalar("commType", "lfm", 2, true);
    m_nHaloCommType = (int)controlDict.readDictScalar("haloCommType", "lfm", 1, true);
    m_bIsDoublePrecision = controlDict.readDictBool("doublePrecision", "lfm", true, true);
    m_bHaveProbes = controlDict.readDictBool("haveProbes", "lfm/post", false, true);
    m_bHaveSampling = controlDict.readDictBool("haveSampling", "lfm/post", false, true);
    m_bHaveAverage = controlDict.readDictBool("haveAverage", "lfm/post", false, true);
    m_tStartAverage = controlDict.readDictScalar("tStartAverage", "lfm/post", 0, true);
    m_bHaveForces = controlDict.readDictBool("haveForces", "lfm/post", false, true);
    m_bHaveResidual = controlDict.readDictBool("haveResiduals", "lfm/post", false, true);
    m_nSaveForcesSteps = (int)controlDict.readDictScalar("saveForcesStep", "lfm/post", 1, true);
    m_nPrintInfoFrequency = (int)controlDict.readDictScalar("printInfoFreq", "lfm/post", 1, true);
    m_bSaveResiduals = controlDict.readDictBool("saveResiduals", "lfm/post", false, true);
    m_bSaveBlendFactor = controlDict.readDictBool("saveBlendFactor", "lfm/post", false, true);
    m_bSaveRank = controlDict.readDictBool("saveRank", "lfm/post", false, true);
    m_bSaveCellOrder = controlDict.readDictBool("saveCellOrder", "lfm/post", false, true);
    m_dCFLMax = controlDict.readDictScalar("maxCo", "", 1, true);

    CDictReaderOF fvScheme("fvSchemes", sys);
    m_nSolver = (int)fvScheme.readDictScalar("solver", "lfm", 0, true);
    m_nDimension = (int)fvScheme.readDictScalar("dimension", "lfm", 2, true);
    m_nRkStepCount = (int)fvScheme.readDictScalar("rkOrder", "lfm", 5, true);
    m_bMinmodInterpolation = fvScheme.readDictBool("minmodExists", "lfm", false, true);
    m_bConstantTimeStep = fvScheme.readDictBool("constantTimeStep", "lfm", true, true);

    CDictReaderOF spongeDict("spongeDict", cst);
    m_dPInf = spongeDict.readDictScalar("pinf");
    m_dTInf = spongeDict.readDictScalar("Tinf");
    m_dUInf[0] = spongeDict.readDictScalar("Uinf_x", "", 0, true);
    m_dUInf[1] = spongeDict.readDictScalar("Uinf_y", "", 0, true);
    m_dUInf[2] = spongeDict.readDictScalar("Uinf_z", "", 0, true);
    m_dLs = spongeDict.readDictScalar("Ls");
    m_dMach = spongeDict.readDictScalar("M");
    m_dK = spongeDict.readDictScalar("k", "", 4.34294481903252e-01, true);

    CDictReaderOF thermo("thermophysicalProperties", cst);
    m_dCp = thermo.readDictScalar("Cp", "mixture/thermodynamics");
    m_dMolWeight = thermo.readDictScalar("molWeight", "mixture/specie");
    m_dMu0 = thermo.readDictScalar("mu", "mixture/transport");
    m_dPrandtl = thermo.readDictScalar("Pr", "mixture/transport");

    CDictReaderOF turbulence("turbulenceProperties", cst);
    m_bisLaminar = turbulence.readDictString("simulationType") == "laminar";
}

bool CInputReader::initialize(int argc, char* argv[]) {
    m_bParallel = false;
    readCase(".");
    return readRuntimeArgs(argc, argv);
}

void CInputReader::showUsage(char* argv[]) {
    std::cerr << "Usage: " << argv[0] << " <option(s)>\n"
              << "Options:\n"
              << "\t-h,--help             Show this help message\n"
              << "\t-p,--parallel         Run the case of processor<rank>\n"
              << "\t-c,--comm_type TYPE   Halo transport (onesided_nonb, onesided_blck, twosided_nonb,\n"
              << "\t                      twosided_blck, twosided_pers, neighcoll_nonb, neighcoll_blck,\n"
              << "\t                      neighcoll_pers); accepted for compatibility, one GPU has no halo "
                 "transport\n"
              << "Case data: constant/polyMesh, system/{controlDict,fvSchemes},\n"
              << "constant/{spongeDict,thermophysicalProperties,turbulenceProperties}\n"
              << std::endl;
}

bool CInputReader::parseHaloCommType(const char* s) {
    static const char* names[] = {"twosided_blck", "twosided_nonb", "twosided_pers", "onesided_blck",
                                  "onesided_nonb", "onesided_pers", "neighcoll_blck", "neighcoll_nonb",
                                  "neighcoll_pers"};
    for (int i = 0; i < 9; ++i)
        if (std::strcmp(s, names[i]) == 0 && i != 5) {
            m_nHaloCommType = i;
            return true;
        }
    return false;
}

bool CInputReader::readRuntimeArgs(int argc, char* argv[]) {
    if (argc < 2) return true;
    static struct option longOptions[] = {{"help", no_argument, 0, 'h'},
                                          {"parallel", no_argument, 0, 'p'},
                                          {"comm_type", required_argument, 0, 'c'},
                                          {0, 0, 0, 0}};
    optind = 1;
    while (true) {
        int idx = 0;
        const int c = getopt_long(argc, argv, "hpc:", longOptions, &idx);
        if (c == -1) break;
        switch (c) {
            case 'h':
                showUsage(argv);
                return false;
            case 'p':
                m_bParallel = true;
                break;
            case 'c':
                if (!parseHaloCommType(optarg)) {
                    std::cerr << "unknown communicator type: " << optarg << std::endl;
                    showUsage(argv);
                    return false;
                }
                break;
            default:
                showUsage(argv);
                return false;
        }
    }
    if (optind < argc) {
        std::printf("non-option ARGV-elements: ");
        while (optind < argc) std::printf("%s ", argv[optind++]);
        std::printf("\n");
    }
    return true;
}
