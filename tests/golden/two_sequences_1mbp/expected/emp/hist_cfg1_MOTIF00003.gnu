set output "hist_cfg1_MOTIF00003.ps"
set key autotitle columnhead
set terminal postscript landscape
set terminal postscript noenhanced
set xrange [-54.5285:15.0417]
set yrange [0:2211]
set xlabel 'PWM score'
set ylabel 'count'
plot "hist_cfg1_MOTIF00003.dat" using 1:2 title 'MOTIF00003 (cfg1)' with boxes
