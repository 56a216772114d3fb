#pragma once
#include <PapillonNDL/stub_common.hpp>
