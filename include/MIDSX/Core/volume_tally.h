// volume_tally.h - volume tallies (reference: include/MIDSX/Core/volume_tally.h).
//
// Geometry and quantities as in the reference; the per-step traversal classification
// (src/MIDSX/Core/volume_tally.cpp:38-91) runs inside the transport kernel.  describe()
// returns the C ABI spec the kernel consumes; a VolumeTally subclass that the GPU does not
// implement throws std::invalid_argument from there (there is no CPU fallback).
#pragma once
#include "../../midsx_gpu.h"
#include "vec3.h"
#include "volume_quantity_container.h"

class VolumeTally {
public:
    virtual ~VolumeTally() = default;
    VolumeQuantityContainer& getVolumeQuantityContainer() { return quantities_; }
    virtual midsx_tally_spec describe() const;

protected:
    VolumeQuantityContainer quantities_;
};

class AACuboidVolumeTally : public VolumeTally {
public:
    AACuboidVolumeTally(Vec3 min_corner, Vec3 max_corner, const VolumeQuantityContainer& quantities);
    midsx_tally_spec describe() const override;
    const Vec3& getMinCorner() const { return min_corner_; }
    const Vec3& getMaxCorner() const { return max_corner_; }

private:
    Vec3 min_corner_;
    Vec3 max_corner_;
};
