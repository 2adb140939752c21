// forwarding header of the glm-subset shim (oracle build only)
#include <glm/glm.hpp>
