#pragma once
#include <map>
#include <string>
namespace exanb {
using ParticleTypeMap = std::map<std::string, int>;
}
// exaDEM's headers name it unqualified (exaNBody's own headers make it visible there)
namespace exaDEM {
using exanb::ParticleTypeMap;
}
