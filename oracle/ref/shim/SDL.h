/* Headless stand-in for the two SDL2 structs the swegl render path touches
 * (SDL_Surface::pixels/pitch/w/h/format->BytesPerPixel).  Test infrastructure
 * for building the reference oracle; no SDL code is involved. */
#pragma once
#include <stdint.h>
typedef struct SDL_PixelFormat { uint8_t BytesPerPixel; } SDL_PixelFormat;
typedef struct SDL_Surface {
    int w, h;
    int pitch;
    void *pixels;
    SDL_PixelFormat *format;
} SDL_Surface;
