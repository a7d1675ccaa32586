// Reconstruction classes of the reference's API, running on the GPU through
// the C ABI (include/muto_gb300.h):
//   MutoVReconstruction   include/MutoVReconstruction.h:11-16
//   MutoPoCA(json)        include/MutoPoCA.h:17-50
//   MutoPoCut(json)       include/MutoPoCut.h:13-28 (derives from MutoPoCA)
//   MutoSLR(json)         include/MutoSLR.h:13-41
//   MutoSLRIter(json)     include/MutoSLRIter.h:9-23 (derives from MutoSLR)
//   MutoMLSD(json)        include/MutoMLSD.h:27-107
//   MutoMAP(json)         include/MutoMAP.h:16-63 (derives from MutoMLSD)
// Constructors take the method's JSON object with the reference's keys and
// defaults.  Errors are printed (as the reference does) and reconstruct()
// then returns an empty image; status() has the counters and the last error.
#pragma once

#include <chrono>
#include <string>

#include "MutoConfig.h"
#include "MutoTypes.h"
#include "muto_gb300.h"

class MutoVReconstruction {
public:
    MutoVReconstruction() {}
    virtual ~MutoVReconstruction() {}
    virtual Image reconstruct(const MutoMuonData&) = 0;
};

// Common part: one library handle per object (not copyable).
class MutoGpuReconstruction : public MutoVReconstruction {
public:
    ~MutoGpuReconstruction() override;
    MutoGpuReconstruction(const MutoGpuReconstruction&) = delete;
    MutoGpuReconstruction& operator=(const MutoGpuReconstruction&) = delete;

    VoxelGrid getCurrentGrid() const;
    muto_status status() const;
    bool ok() const { return fHandle != nullptr; }

protected:
    MutoGpuReconstruction(const char* method, const json& config);
    Image reconstructOnce(const MutoMuonData& rays);  // load, prepare (the whole method), image
    Image fetchImage();
    bool check(int rc, const char* what);
    void logMessage(const std::string& msg, bool printTime = false);

    muto_handle* fHandle = nullptr;
    json fConfig;
    std::string fMethod;
    bool fLogPrint = false;
    std::chrono::steady_clock::time_point fTimeStart;
};

class MutoPoCA : public MutoGpuReconstruction {
public:
    MutoPoCA();
    explicit MutoPoCA(json config);
    Image reconstruct(const MutoMuonData& rays) override;

protected:
    MutoPoCA(const char* method, json config);
};

// PoCA keeping, per voxel, the lowest cut_percentile of the scattering values
class MutoPoCut : public MutoPoCA {
public:
    MutoPoCut();
    explicit MutoPoCut(json config);
};

// straight-line back-projection between the grid's top and bottom planes
// (a MutoVReconstruction of its own, as include/MutoSLR.h:13 declares it)
class MutoSLR : public MutoGpuReconstruction {
public:
    MutoSLR();
    explicit MutoSLR(json config);
    Image reconstruct(const MutoMuonData& rays) override;

protected:
    MutoSLR(const char* method, json config);
};

// SLR repeated num_iteration times, later passes in place in muon order
class MutoSLRIter : public MutoSLR {
public:
    MutoSLRIter();
    explicit MutoSLRIter(json config);
};

class MutoMLSD : public MutoGpuReconstruction {
public:
    MutoMLSD();
    explicit MutoMLSD(json config);
    Image reconstruct(const MutoMuonData& rays) override;

protected:
    MutoMLSD(const char* method, json config);
    int fNIteration = 10;
};

class MutoMAP : public MutoMLSD {
public:
    MutoMAP();
    explicit MutoMAP(json config);
};
