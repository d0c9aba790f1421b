/*
 * Tape (API call record/replay) entry points, declared with the signatures of RobotecGPULidar's
 * include/rgl/api/extensions/tape.h:26-45 so that plugins linking them still load. Recording and
 * replay are not part of this GB300 build: the calls return RGL_NOT_IMPLEMENTED
 * (rgl_tape_record_is_active reports false).
 */
#pragma once

#include <rgl/api/core.h>

RGL_API rgl_status_t rgl_tape_record_begin(const char* path);
RGL_API rgl_status_t rgl_tape_record_end();
RGL_API rgl_status_t rgl_tape_record_is_active(bool* is_active);
RGL_API rgl_status_t rgl_tape_play(const char* path);
