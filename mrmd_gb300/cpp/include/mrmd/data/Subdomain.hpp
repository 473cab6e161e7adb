// Drop-in data::Subdomain (data/Subdomain.hpp:37-110).
#pragma once

#include "../datatypes.hpp"

namespace mrmd::data
{
struct Subdomain
{
    Subdomain() = default;
    Subdomain(const Point3D& minCornerArg, const Point3D& maxCornerArg, const Vector3D& ghostLayerThicknessArg)
    {
        gb300::check(mrmd_subdomain_init(&s, minCornerArg.data(), maxCornerArg.data(), ghostLayerThicknessArg.data()),
                    "Subdomain");
        for (int d = 0; d < 3; ++d)
        {
            minCorner[d] = s.minCorner[d];
            maxCorner[d] = s.maxCorner[d];
            ghostLayerThickness[d] = s.ghostLayerThickness[d];
            minGhostCorner[d] = s.minGhostCorner[d];
            maxGhostCorner[d] = s.maxGhostCorner[d];
            minInnerCorner[d] = s.minInnerCorner[d];
            maxInnerCorner[d] = s.maxInnerCorner[d];
            diameter[d] = s.diameter[d];
            diameterWithGhostLayer[d] = s.diameterWithGhostLayer[d];
        }
    }
    Subdomain(const Point3D& minCornerArg, const Point3D& maxCornerArg, const real_t& ghostLayerThicknessArg)
        : Subdomain(minCornerArg, maxCornerArg,
                    Vector3D{ghostLayerThicknessArg, ghostLayerThicknessArg, ghostLayerThicknessArg})
    {
    }

    real_t getVolume() const { return diameter[0] * diameter[1] * diameter[2]; }
    Point3D getCenter() const
    {
        return {(minCorner[0] + maxCorner[0]) * 0.5, (minCorner[1] + maxCorner[1]) * 0.5,
                (minCorner[2] + maxCorner[2]) * 0.5};
    }

    Point3D minCorner{}, maxCorner{}, ghostLayerThickness{};
    Point3D minGhostCorner{}, maxGhostCorner{}, minInnerCorner{}, maxInnerCorner{};
    Vector3D diameter{}, diameterWithGhostLayer{};
    mrmd_subdomain s{};
};
}  // namespace mrmd::data
