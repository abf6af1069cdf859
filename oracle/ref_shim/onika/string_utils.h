#pragma once
#include <string>
