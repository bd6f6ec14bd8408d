/* Test infrastructure (oracle only): headless stand-in for freeglut.  The three
 * constants compared outside a call (main.cpp:383, :409, :414) get values; every
 * glut* call is a no-op expression.  Used for OpenCloth_Implicit and
 * OpenCloth_CoRotated_Linear_FEM. */
#ifndef OC_SHIM_FREEGLUT_H
#define OC_SHIM_FREEGLUT_H
#include "glew.h"
#define GLUT_DOWN 0
#define GLUT_UP 1
#define GLUT_MIDDLE_BUTTON 1
#define glutInit(...) (0)
#define glutInitDisplayMode(...) (0)
#define glutInitWindowSize(...) (0)
#define glutCreateWindow(...) (0)
#define glutDisplayFunc(...) (0)
#define glutReshapeFunc(...) (0)
#define glutIdleFunc(...) (0)
#define glutMouseFunc(...) (0)
#define glutMotionFunc(...) (0)
#define glutCloseFunc(...) (0)
#define glutMainLoop(...) (0)
#define glutGet(...) (0)
#define glutSetCursor(...) (0)
#define glutPostRedisplay(...) (0)
#define glutSetWindowTitle(...) (0)
#define glutSwapBuffers(...) (0)
#define glutWireSphere(...) (0)
#define glutKeyboardFunc(...) (0)
#endif
