/* empty stand-in: the reference includes this header but uses nothing from it on the hashing path */
#include "sha.h"
