/* config.h -- what CMake's configure_file writes from config.h.in
 * (project relxill VERSION 2.4, CMakeLists.txt:3). */
#ifndef CONFIG_H_IN_
#define CONFIG_H_IN_
#define PROJECT_NAME "relxill"
#define PROJECT_VER "2.4"
#define PROJECT_VER_MAJOR "2"
#define PROJECT_VER_MINOR "4"
#define PROJECT_VER_PATCH ""
#endif
