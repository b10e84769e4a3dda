/* Headless stand-in for <GL/glut.h> (oracle build only). */
#include <GL/gl.h>
