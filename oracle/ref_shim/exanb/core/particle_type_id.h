#pragma once
#include <map>
#include <string>
namespace exanb {
using ParticleTypeMap = std::map<std::string, int>;
}
