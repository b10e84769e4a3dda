/* Headless stand-in for <GL/glu.h> (oracle build only). */
#include <GL/gl.h>
