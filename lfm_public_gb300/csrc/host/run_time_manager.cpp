// CRunTimeManagerOF without OpenFOAM.
//
// Follows runTimeManagerOF/runTimeManagerOF.cpp: the case is "." or
// "processor<rank>" under the working directory (:5-13); every accessor reads
// the Foam::Time state (restated by lfm::FoamTime): run() is
// time < endTime - deltaT/2, ++ advances one deltaT and sets the write flag from
// writeControl/writeInterval, write() writes every AUTO_WRITE field of the case
// into the current time directory (:48-109).
#include "runTimeManagerOF.h"

#include <string>

#include "foam_case.h"

CRunTimeManagerOF::CRunTimeManagerOF(const int nRank) {
    const std::string caseName = (nRank >= 0) ? "processor" + std::to_string(nRank) : ".";
    m_pRunTime = lfm::newFoamTime(".", caseName);
}

CRunTimeManagerOF::~CRunTimeManagerOF() { delete static_cast<lfm::FoamTime*>(m_pRunTime); }

static lfm::FoamTime& T(void* p) { return *static_cast<lfm::FoamTime*>(p); }

double CRunTimeManagerOF::getStartTime() const { return T(m_pRunTime).startTime; }
double CRunTimeManagerOF::getEndTime() const { return T(m_pRunTime).endTime; }
double CRunTimeManagerOF::getCurrentTime() const { return T(m_pRunTime).value; }
double CRunTimeManagerOF::getDeltaTime() const { return T(m_pRunTime).deltaT; }
void CRunTimeManagerOF::setDeltaTime(const double dDeltaTime) { T(m_pRunTime).deltaT = dDeltaTime; }
bool CRunTimeManagerOF::isAdjustDeltaTime() const { return T(m_pRunTime).adjustTimeStep; }
int CRunTimeManagerOF::getTimeStep() const { return (int)T(m_pRunTime).timeIndex; }
void CRunTimeManagerOF::advanceTime() { T(m_pRunTime).increment(); }
bool CRunTimeManagerOF::isRunning() { return T(m_pRunTime).running(); }
bool CRunTimeManagerOF::isWriteTime() { return T(m_pRunTime).writeTime; }
void CRunTimeManagerOF::writeResults() { T(m_pRunTime).write(); }
