#pragma once
#include <Minuit2/FCNBase.h>
