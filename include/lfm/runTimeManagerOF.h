// CRunTimeManagerOF without OpenFOAM: controlDict-driven time loop and field
// output for case "." or "processor<rank>". Same class as the reference's
// api/runTimeManagerOF.h:9-51.
#ifndef LFM_RUN_TIME_MANAGER_OF_H
#define LFM_RUN_TIME_MANAGER_OF_H

#include "runTimeManager.h"

class CRunTimeManagerOF : public IRunTimeManager {
public:
    CRunTimeManagerOF(const int nRank);
    virtual ~CRunTimeManagerOF();

    virtual double getStartTime() const;
    virtual double getEndTime() const;
    virtual double getCurrentTime() const;

    virtual double getDeltaTime() const;
    virtual void setDeltaTime(const double dDeltaTime);
    virtual bool isAdjustDeltaTime() const;

    virtual int getTimeStep() const;
    virtual void advanceTime();

    virtual bool isRunning();
    virtual bool isWriteTime();
    virtual void writeResults();

    virtual void* getRunPointer() { return m_pRunTime; }

protected:
    void* m_pRunTime;
};

#endif
