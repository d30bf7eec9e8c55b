// Stand-in: the reference's estimator.h includes core/film.h but StatTile needs nothing from it.
#pragma once
