set output "hist_cfg1_MOTIF00001.ps"
set key autotitle columnhead
set terminal postscript landscape
set terminal postscript noenhanced
set xrange [-89.2101:27.4185]
set yrange [0:192758]
set xlabel 'PWM score'
set ylabel 'count'
plot "hist_cfg1_MOTIF00001.dat" using 1:2 title 'MOTIF00001 (cfg1)' with boxes
