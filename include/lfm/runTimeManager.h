// IRunTimeManager: time control and result output. Same interface as the
// reference's api/runTimeManager.h:7-44.
#ifndef LFM_RUN_TIME_MANAGER_H
#define LFM_RUN_TIME_MANAGER_H

class IRunTimeManager {
public:
    virtual ~IRunTimeManager() {}

    virtual double getStartTime() const = 0;
    virtual double getEndTime() const = 0;
    virtual double getCurrentTime() const = 0;

    virtual double getDeltaTime() const = 0;
    virtual void setDeltaTime(const double dDeltaTime) = 0;
    virtual bool isAdjustDeltaTime() const = 0;

    virtual int getTimeStep() const = 0;
    virtual void advanceTime() = 0;

    virtual bool isRunning() = 0;
    virtual bool isWriteTime() = 0;
    virtual void writeResults() = 0;

    virtual void* getRunPointer() = 0;
};

#endif
