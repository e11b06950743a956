#pragma once
#include <parsec.h>
