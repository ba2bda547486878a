/* Headless stand-in: WGL is not used by the reference step. */
#pragma once
