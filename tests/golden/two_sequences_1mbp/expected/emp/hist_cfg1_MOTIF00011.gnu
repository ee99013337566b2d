set output "hist_cfg1_MOTIF00011.ps"
set key autotitle columnhead
set terminal postscript landscape
set terminal postscript noenhanced
set xrange [-79.5396:23.8226]
set yrange [0:2630]
set xlabel 'PWM score'
set ylabel 'count'
plot "hist_cfg1_MOTIF00011.dat" using 1:2 title 'MOTIF00011 (cfg1)' with boxes
