#pragma once
#include <sys/stat.h>
#define _mkdir(p) mkdir((p), 0755)
