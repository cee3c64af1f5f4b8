/* Empty stand-in for libtiff's header: the reference's engine includes it
 * (FBPG/mucat_file.h:9) without using it. */
#pragma once
