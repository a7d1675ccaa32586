// Muon data and image files (the reference's include/MutoFile.h:27-68).
//
//   getMuonData     raw detector hits -> tracks (src/MutoFile.cpp:19-82, :248-304)
//   saveImage       64-byte header + column-major f32/f64 image (:85-133)
//   saveImagePure   the image alone (:136-157)
//   loadImage       header + image (:160-211)
//   loadImagePure   the image alone, grid given (:214-245)
//   getCurrentPath  the start-up working directory (include/MutoFile.h:65)
#pragma once

#include <string>
#include <utility>
#include <vector>

#include "MutoTypes.h"

class MutoFile {
public:
    // Reads records of 2*zlayers.size()+2 values (f32 when fPrecision is 4,
    // f64 when 8): {ein, x0, y0, ..., x_{n-1}, y_{n-1}, eout}.  Records with a
    // NaN are skipped.  The first nMiddle layers give the incoming line, the
    // rest the outgoing one: each line is the principal axis of its hits (the
    // direction the reference takes from a thin SVD), oriented with d_z > 0;
    // pin lies on layer nMiddle-1, pout on layer nMiddle.
    static MutoMuonData getMuonData(std::vector<std::string> flist, std::vector<MTfloat> zlayers, int nMiddle,
                                    int fPrecision = 4);
    static bool saveImage(const Image& img, const ImageHeader& header, std::string filename);
    static bool saveImagePure(const Image& img, std::string filename, MTindex fPrecision = 4);
    // A file that cannot be read gives an empty image (size() == 0).
    static std::pair<Image, ImageHeader> loadImage(std::string filename);
    static Image loadImagePure(std::string filename, VoxelGrid grid, MTindex fPrecision = 4);

    // The working directory when the library was loaded (the reference keeps
    // it in a static member set at start-up, src/MutoFile.cpp:11-15).
    static std::string getCurrentPath();

    // One line fit of getMuonData: centroid and unit direction (d_z >= 0) of
    // n points.
    static void fitLine(const double* x, const double* y, const double* z, int n, double* centroid, double* dir);
};
